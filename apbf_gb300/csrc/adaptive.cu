// adaptive.cu -- the adaptive stages: split/merge decisions and claims, split
// duplication, particle transfer with list compaction, kernel-width spreading.
// Compiled with -fmad=false: the decisions are plain FP32 arithmetic and must be
// bit-identical to the oracle's exact FP32 emulation.
//
//  update_transfers::apply (source/update_transfers.cpp:14-71)
//    k_fsm12     find_split_and_merge_1.comp + _2.comp as one gather over each row
//                (integer fixed-point distances, smallest-index tie)
//    k_fsm3      find_split_and_merge_3.comp:46-92: target radius, boundary-distance
//                decay, split / merge proposals
//    k_compact*  proposals in particle-index order (stable scan compaction)
//    k_claims    one CTA resolves the claims of find_split_and_merge_3.comp:94-121 in
//                particle-index order (rounds of "smallest undecided claimant wins",
//                exactly the sequential result) and applies the capacity limits of
//                :103-119 and remove_impossible_splits.comp:29-45
//    k_split     indexed_list::duplicate_these (indexed_list.h:140-152) +
//                initialize_split_particles.comp:18-32
//  particle_transfer::apply (source/particle_transfer.cpp:10-28)
//    k_transfer  particle_transfer.comp:31-85
//    k_compact_* delete_these (indexed_list.h:125-138) for transfers and particles
//  spread_kernel_width::apply (source/spread_kernel_width.cpp:12-26)
//    k_kw_init, k_kw_spread, k_kw_gradual
#include "apbf_internal.cuh"

namespace apbf {
namespace {

// floor(sqrt(x)) exactly: FP32 estimate, then integer correction.
__device__ __forceinline__ uint32_t isqrt_u64(unsigned long long x) {
    unsigned long long r = (unsigned long long)sqrtf((float)x);
    while (r > 0 && r * r > x) --r;
    while ((r + 1) * (r + 1) <= x) ++r;
    return (uint32_t)r;
}

__device__ __forceinline__ uint32_t fixed_dist(int4 a, int4 b) {
    long long dx = (long long)b.x - a.x, dy = (long long)b.y - a.y, dz = (long long)b.z - a.z;
    unsigned long long s = (unsigned long long)(dx * dx) + (unsigned long long)(dy * dy) +
                           (unsigned long long)(dz * dz);
    return isqrt_u64(s);
}

// Proposal encoding: kind in bits 30..31 of pkind, source / target ids separate.
constexpr uint32_t kPropNone = 0u, kPropMerge = 1u, kPropSplit = 2u;

// find_split_and_merge_1 + _2: bd_i = min_j(bd_j + d_ij), d_min_i, nearest_i.
__global__ void k_fsm12(const int4 *__restrict__ pos, const uint32_t *__restrict__ old_bd,
                        uint32_t *__restrict__ new_bd, uint32_t *__restrict__ nearest, const uint32_t *count,
                        const uint32_t *idx, uint32_t stride, const uint32_t *d_len) {
    const uint32_t n = d_len[kLenParticles];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int4 p = pos[i];
        uint32_t bd = 0xffffffffu, md = 0xffffffffu, nn = 0xffffffffu;
        const uint32_t c = count[i];
        const uint32_t *row = idx + i;
        // batches of four neighbours, software-pipelined: a batch's gathers go out with
        // the row entries of the next (the minima do not depend on the order)
        constexpr uint32_t U = 4;
        uint32_t jj[U];
#pragma unroll
        for (uint32_t u = 0; u < U; ++u) jj[u] = u < c ? row[(size_t)u * stride] : i;
        for (uint32_t k0 = 0; k0 < c; k0 += U) {
            int4 q[U];
            uint32_t ob[U], jn[U];
#pragma unroll
            for (uint32_t u = 0; u < U; ++u) {
                q[u] = pos[jj[u]];
                ob[u] = old_bd[jj[u]];
            }
#pragma unroll
            for (uint32_t u = 0; u < U; ++u) {
                const uint32_t k = k0 + U + u;
                jn[u] = k < c ? row[(size_t)k * stride] : i;
            }
#pragma unroll
            for (uint32_t u = 0; u < U; ++u) {
                if (k0 + u >= c) break;
                const uint32_t j = jj[u];
                const uint32_t d = fixed_dist(p, q[u]);
                const uint32_t cand = ob[u] + d;  // uint wrap as in the shader
                bd = cand < bd ? cand : bd;
                if (d < md || (d == md && j < nn)) {
                    md = d;
                    nn = j;
                }
            }
#pragma unroll
            for (uint32_t u = 0; u < U; ++u) jj[u] = jn[u];
        }
        new_bd[i] = bd;
        nearest[i] = nn;
    }
}

struct Fsm3Args {
    FluidBufs f;
    const uint32_t *nearest;
    uint32_t *pkind;  // per particle: proposal kind
    uint32_t *psrc;
    uint32_t *ptgt;
    uint32_t *flag;   // per particle: 1 if it proposes (for the compaction scan)
    const uint32_t *d_len;
    float split_c, sf, rmin, offset;
    int merge, split, update_target, bd_mode;
};

// find_split_and_merge_3.comp:49-92 (everything before the claims).
__global__ void k_fsm3(Fsm3Args a) {
    const uint32_t n = a.d_len[kLenParticles];
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < n; id += gridDim.x * blockDim.x) {
        const int4 p = a.f.pos[id];
        const float radius = a.f.radius[id];
        const float bdist = (float)a.f.boundary_distance[id] / 262144.0f;
        float bness = a.f.boundariness[id];
        const uint32_t nn = a.nearest[id];
        const bool has_nn = nn != 0xffffffffu;
        float nnd = 0.0f, nnr = 0.0f;
        bool nn_larger = false;
        if (has_nn) {
            const int4 q = a.f.pos[nn];
            const float dx = (float)wadd(q.x, -p.x), dy = (float)wadd(q.y, -p.y), dz = (float)wadd(q.z, -p.z);
            nnd = sqrtf((dx * dx + dy * dy) + dz * dz) / 262144.0f;
            nnr = a.f.radius[nn];
            nn_larger = nnr > radius || (nnr == radius && nn > id);
        }
        float target;
        if (a.update_target) {
            if (a.bd_mode) {
                target = (a.sf / (4.0f + 4.0f * a.sf)) * bdist;
                target = fmaxf(target, a.rmin);
            } else {
                target = a.rmin + fmaxf(0.0f, (bdist - a.offset) * a.sf);
            }
            a.f.target_radius[id] = target;
        } else {
            target = a.f.target_radius[id];
        }
        bness = bness >= 1.0f ? 1.0f : 0.0f;
        a.f.boundary_distance[id] = f2u((bdist * (1.0f - bness) + radius * bness) * 262144.0f);
        a.f.boundariness[id] = bness;
        const bool split = a.split && (target * a.split_c <= radius);
        const bool merge = a.merge && has_nn && nnd < radius &&
                           (radius * radius * radius + nnr * nnr * nnr <= target * target * target);
        uint32_t kind = kPropNone;
        if (merge) kind = kPropMerge;
        else if (split) kind = kPropSplit;
        a.pkind[id] = kind;
        a.psrc[id] = (merge && nn_larger) ? nn : id;
        a.ptgt[id] = (merge && nn_larger) ? id : nn;
        a.flag[id] = kind != kPropNone ? 1u : 0u;
    }
}

// Writes the proposing particle ids in index order: list[scan[i]-1] = i.
__global__ void k_compact_ids(const uint32_t *flag, const uint32_t *scan, uint32_t *list, const uint32_t *d_len,
                              uint32_t *count_out) {
    const uint32_t n = d_len[kLenParticles];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (flag[i]) list[scan[i] - 1u] = i;
    if (blockIdx.x == 0 && threadIdx.x == 0) *count_out = n ? scan[n - 1] : 0u;
}

struct ClaimArgs {
    const uint32_t *list;   // proposing particle ids, increasing
    const uint32_t *count;  // number of proposals
    const uint32_t *pkind, *psrc, *ptgt;
    uint32_t *owner;        // per particle scratch, all 0xffffffff on entry and exit
    uint32_t *state;        // per proposal slot
    uint32_t *transferring;
    TransferBufs t;
    uint32_t *d_len;
    uint32_t *splits;       // accepted split ids (output, index order)
    uint32_t max_transfers, particle_cap;
    float merge_ttl, split_ttl;
    Status *st;
};

constexpr uint32_t kUndecided = 0u, kAccepted = 1u, kRejected = 2u;
constexpr int kClaimThreads = 1024;

// One CTA.  Sequential semantics of the claims in particle-index order: a proposal
// is accepted iff none of its particles is transferring (from earlier transfers or
// an earlier accepted proposal).  Each round, every undecided proposal that is the
// smallest undecided claimant of all its particles is decided; so is every
// proposal whose particle was taken.  The smallest undecided proposal is always
// decided, so at most `count` rounds are needed.
__global__ void __launch_bounds__(kClaimThreads) k_claims(ClaimArgs a) {
    __shared__ uint32_t s_left;
    __shared__ uint32_t s_warp[kClaimThreads / 32];
    __shared__ uint32_t s_base;
    const uint32_t m = *a.count;
    const int t = threadIdx.x;
    for (uint32_t k = t; k < m; k += kClaimThreads) a.state[k] = kUndecided;
    __syncthreads();
    for (uint32_t round = 0; round <= m; ++round) {
        if (t == 0) s_left = 0u;
        // phase A: register claims
        for (uint32_t k = t; k < m; k += kClaimThreads) {
            if (a.state[k] != kUndecided) continue;
            const uint32_t id = a.list[k];
            atomicMin(&a.owner[a.psrc[id]], k);
            if (a.pkind[id] == kPropMerge) atomicMin(&a.owner[a.ptgt[id]], k);
        }
        __syncthreads();
        // phase B: decide
        for (uint32_t k = t; k < m; k += kClaimThreads) {
            if (a.state[k] != kUndecided) continue;
            const uint32_t id = a.list[k];
            const bool merge = a.pkind[id] == kPropMerge;
            const uint32_t s = a.psrc[id], g = a.ptgt[id];
            const bool taken = ((volatile uint32_t *)a.transferring)[s] != 0u ||
                               (merge && ((volatile uint32_t *)a.transferring)[g] != 0u);
            if (taken) {
                a.state[k] = kRejected;
            } else if (a.owner[s] == k && (!merge || a.owner[g] == k)) {
                a.state[k] = kAccepted;
                a.transferring[s] = 1u;
                if (merge) a.transferring[g] = 1u;
            } else {
                s_left = 1u;
            }
        }
        __syncthreads();
        // phase C: reset the owners
        for (uint32_t k = t; k < m; k += kClaimThreads) {
            const uint32_t id = a.list[k];
            a.owner[a.psrc[id]] = 0xffffffffu;
            if (a.pkind[id] == kPropMerge) a.owner[a.ptgt[id]] = 0xffffffffu;
        }
        __syncthreads();
        if (s_left == 0u) break;
        __syncthreads();
    }
    // capacity (C7): accepted merges in index order up to the free transfers, then
    // accepted splits up to the transfers and particles still free
    const uint32_t n = a.d_len[kLenParticles];
    const uint32_t t0 = a.d_len[kLenTransfers];
    const uint32_t room_t = a.max_transfers > t0 ? a.max_transfers - t0 : 0u;
    for (int pass = 0; pass < 2; ++pass) {
        const uint32_t want = pass == 0 ? kPropMerge : kPropSplit;
        if (t == 0) s_base = 0u;
        __syncthreads();
        for (uint32_t k0 = 0; k0 < m; k0 += kClaimThreads) {
            const uint32_t k = k0 + t;
            bool mine = false;
            uint32_t id = 0;
            if (k < m) {
                id = a.list[k];
                mine = a.state[k] == kAccepted && a.pkind[id] == want;
            }
            // block-wide exclusive rank of this chunk's accepted proposals
            const uint32_t bal = __ballot_sync(0xffffffffu, mine);
            const uint32_t lane = t & 31, w = t >> 5;
            if (lane == 0) s_warp[w] = __popc(bal);
            __syncthreads();
            if (t == 0) {
                uint32_t run = s_base;
                for (int x = 0; x < kClaimThreads / 32; ++x) {
                    uint32_t c = s_warp[x];
                    s_warp[x] = run;
                    run += c;
                }
                s_base = run;
            }
            __syncthreads();
            const uint32_t rank = s_warp[w] + __popc(bal & ((1u << lane) - 1u));
            if (mine) {
                const uint32_t s = a.psrc[id];
                if (want == kPropMerge) {
                    if (rank < room_t) {
                        a.t.source[t0 + rank] = s;
                        a.t.target[t0 + rank] = a.ptgt[id];
                        a.t.time_left[t0 + rank] = a.merge_ttl;
                    } else {
                        a.transferring[s] = 0u;
                        a.transferring[a.ptgt[id]] = 0u;
                        set_flag(a.st, APBF_FLAG_TRANSFER_OVERFLOW);
                    }
                } else {
                    a.splits[rank] = id;
                }
            }
            __syncthreads();
        }
        if (pass == 0) {
            __syncthreads();
            const uint32_t merges = s_base < room_t ? s_base : room_t;
            if (t == 0) {
                if (s_base > room_t) atomicMax(&a.st->required_transfers, t0 + s_base);
                a.d_len[kLenMerges] = merges;
            }
            __syncthreads();
        }
    }
    __syncthreads();
    // remove_impossible_splits.comp:34-44
    const uint32_t nt = t0 + a.d_len[kLenMerges];
    const uint32_t free_t = a.max_transfers > nt ? a.max_transfers - nt : 0u;
    const uint32_t free_p = a.particle_cap > n ? a.particle_cap - n : 0u;
    const uint32_t ns = s_base;
    uint32_t keep = ns < free_t ? ns : free_t;
    keep = keep < free_p ? keep : free_p;
    for (uint32_t k = keep + t; k < ns; k += kClaimThreads) a.transferring[a.splits[k]] = 0u;
    for (uint32_t k = t; k < keep; k += kClaimThreads) {
        a.t.source[nt + k] = a.splits[k];
        a.t.target[nt + k] = n + k;
        a.t.time_left[nt + k] = a.split_ttl;
    }
    __syncthreads();
    if (t == 0) {
        if (keep < ns) {
            set_flag(a.st, keep < free_p ? APBF_FLAG_TRANSFER_OVERFLOW : APBF_FLAG_PARTICLE_OVERFLOW);
            atomicMax(&a.st->required_particles, n + ns);
        }
        a.d_len[kLenSplits] = keep;
        a.d_len[kLenTransfers] = nt + keep;
    }
}

// duplicate_these + initialize_split_particles: slot n + k copies split k.
__global__ void k_split(FluidBufs f, const uint32_t *splits, uint32_t *d_len) {
    const uint32_t n = d_len[kLenParticles], ns = d_len[kLenSplits];
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < ns; k += gridDim.x * blockDim.x) {
        const uint32_t s = splits[k], d = n + k;
        const float r = f.radius[s];
        int4 p = f.pos[s];
        p.x = wadd(p.x, f2i((r * 262144.0f) * 0.1f));
        f.pos[d] = p;
        f.vel[d] = f.vel[s];
        f.inv_mass[d] = __int_as_float(0x7f800000);  // 1/0 (C9)
        f.radius[d] = 0.0f;
        f.pos_backup[d] = f.pos_backup[s];
        f.transferring[d] = f.transferring[s];
        f.target_radius[d] = f.target_radius[s];
        f.kernel_width[d] = f.kernel_width[s];
        f.boundariness[d] = f.boundariness[s];
        f.lambda_prev[d] = f.lambda_prev[s];
        f.boundary_distance[d] = f.boundary_distance[s];
    }
}

__global__ void k_split_len(uint32_t *d_len) { d_len[kLenParticles] += d_len[kLenSplits]; }

// particle_transfer.comp:31-85 with C9 for split targets.
__global__ void k_transfer(FluidBufs f, TransferBufs t, uint32_t *pdel, uint32_t *tkeep, const uint32_t *d_len,
                           float dt) {
    const uint32_t nt = d_len[kLenTransfers];
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < nt; id += gridDim.x * blockDim.x) {
        const float tt = t.time_left[id];
        const float ttl = fmaxf(dt, fabsf(tt));
        const bool merge = tt > 0.0f;
        const uint32_t S = t.source[id], T = t.target[id];
        const float rS = f.radius[S], rT = f.radius[T];
        const float imS = f.inv_mass[S], imT = f.inv_mass[T];
        const float volS = rS * rS * rS, volT = rT * rT * rT;
        const float factor = merge ? fminf(1.0f, dt / ttl) : dt * (volS - volT) / (2.0f * ttl * volS);
        const float tv = factor * volS;
        f.inv_mass[S] = imS / (1.0f - factor);
        f.inv_mass[T] = isinf(imT) ? imS / factor : imS * imT * (1.0f / (imS + factor * imT));
        f.radius[S] = cbrtf(volS - tv);
        f.radius[T] = cbrtf(volT + tv);
        t.time_left[id] = (ttl - dt) * (merge ? 1.0f : -1.0f);
        uint32_t keep = 1u;
        if (ttl == dt) {
            if (merge) pdel[S] = 1u;  // the merged source particle is deleted; its transfer with it
            keep = 0u;
            f.transferring[S] = 0u;
            f.transferring[T] = 0u;
        }
        tkeep[id] = keep;
    }
}

__global__ void k_keep_flags(const uint32_t *pdel, uint32_t *pkeep, const uint32_t *d_len) {
    const uint32_t n = d_len[kLenParticles];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        pkeep[i] = pdel[i] ? 0u : 1u;
}

// Stable compaction of the particles: new index = scan[i] - 1 for kept i.
__global__ void k_compact_particles(FluidBufs src, FluidBufs dst, const uint32_t *scan, const uint32_t *pdel,
                                    const uint32_t *d_len) {
    const uint32_t n = d_len[kLenParticles];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (pdel[i]) continue;
        const uint32_t k = scan[i] - 1u;
        dst.pos[k] = src.pos[i];
        dst.vel[k] = src.vel[i];
        dst.inv_mass[k] = src.inv_mass[i];
        dst.radius[k] = src.radius[i];
        dst.pos_backup[k] = src.pos_backup[i];
        dst.transferring[k] = src.transferring[i];
        dst.target_radius[k] = src.target_radius[i];
        dst.kernel_width[k] = src.kernel_width[i];
        dst.boundariness[k] = src.boundariness[i];
        dst.lambda_prev[k] = src.lambda_prev[i];
        dst.boundary_distance[k] = src.boundary_distance[i];
    }
}

// Transfers survive if kept and neither particle was deleted; ids follow the
// particle compaction (indexed_list.h:288-308).
__global__ void k_transfer_keep2(const TransferBufs t, uint32_t *tkeep, const uint32_t *pdel, const uint32_t *d_len) {
    const uint32_t nt = d_len[kLenTransfers];
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < nt; id += gridDim.x * blockDim.x)
        if (pdel[t.source[id]] || pdel[t.target[id]]) tkeep[id] = 0u;
}

__global__ void k_compact_transfers(TransferBufs src, TransferBufs dst, const uint32_t *tkeep,
                                    const uint32_t *tscan, const uint32_t *pscan, const uint32_t *d_len) {
    const uint32_t nt = d_len[kLenTransfers];
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < nt; id += gridDim.x * blockDim.x) {
        if (!tkeep[id]) continue;
        const uint32_t k = tscan[id] - 1u;
        dst.source[k] = pscan[src.source[id]] - 1u;
        dst.target[k] = pscan[src.target[id]] - 1u;
        dst.time_left[k] = src.time_left[id];
    }
}

__global__ void k_compact_lengths(const uint32_t *pscan, const uint32_t *tscan, uint32_t *d_len) {
    const uint32_t n = d_len[kLenParticles], nt = d_len[kLenTransfers];
    d_len[kLenParticles] = n ? pscan[n - 1] : 0u;
    d_len[kLenTransfers] = nt ? tscan[nt - 1] : 0u;
}

// kernel_width_init.comp:21-36
__global__ void k_kw_init(FluidBufs f, uint32_t *ukw, const uint32_t *d_len, int use_target) {
    const uint32_t n = d_len[kLenParticles];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float tr = use_target ? f.target_radius[i] : 0.0f;
        ukw[i] = f2u(fmaxf(f.radius[i], tr) * 4.0f * 262144.0f);
    }
}

// kernel_width.comp:26-61: spread (atomicMax) and prune row i in place, order kept.
__global__ void k_kw_spread(FluidBufs f, uint32_t *ukw, uint32_t *count, uint32_t *idx, uint32_t stride,
                            const uint32_t *d_len, int use_target) {
    const uint32_t n = d_len[kLenParticles];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int4 p = f.pos[i];
        const float tr = use_target ? f.target_radius[i] : 0.0f;
        const float ok = fmaxf(f.radius[i], tr) * 4.0f;
        const float cut = fmaxf(ok, f.kernel_width[i]);
        const uint32_t c = count[i];
        uint32_t w = 0;
        // batches of four neighbours, software-pipelined (the pruned row is written
        // behind the entries read ahead); a maximum only grows, so an atomic whose value
        // a plain read already meets or exceeds would change nothing and is left out
        constexpr uint32_t U = 4;
        uint32_t *row = idx + i;
        uint32_t jj[U];
#pragma unroll
        for (uint32_t u = 0; u < U; ++u) jj[u] = u < c ? row[(size_t)u * stride] : i;
        for (uint32_t k0 = 0; k0 < c; k0 += U) {
            int4 q[U];
            uint32_t cur[U], jn[U];
#pragma unroll
            for (uint32_t u = 0; u < U; ++u) {
                q[u] = f.pos[jj[u]];
                cur[u] = *(volatile const uint32_t *)&ukw[jj[u]];
            }
#pragma unroll
            for (uint32_t u = 0; u < U; ++u) {
                const uint32_t k = k0 + U + u;
                jn[u] = k < c ? row[(size_t)k * stride] : i;
            }
#pragma unroll
            for (uint32_t u = 0; u < U; ++u) {
                if (k0 + u >= c) break;
                const uint32_t j = jj[u];
                const float dx = (float)wadd(q[u].x, -p.x) / 262144.0f, dy = (float)wadd(q[u].y, -p.y) / 262144.0f,
                            dz = (float)wadd(q[u].z, -p.z) / 262144.0f;
                const float dist = sqrtf((dx * dx + dy * dy) + dz * dz);
                const float infl = fmaxf(0.0f, 1.0f - fmaxf(0.0f, (dist - ok) / (ok * 0.5f)));
                const uint32_t v = f2u((ok * infl) * 262144.0f);
                if (v > cur[u]) atomicMax(&ukw[j], v);
                if (dist <= cut) row[(size_t)(w++) * stride] = j;
            }
#pragma unroll
            for (uint32_t u = 0; u < U; ++u) jj[u] = jn[u];
        }
        count[i] = w;
    }
}

__device__ __forceinline__ float move_towards_geo(float old_v, float new_v, float step) {
    float dir = new_v > old_v ? 1.0f : (new_v < old_v ? -1.0f : 0.0f);
    float result = old_v * (1.0f + step * dir);
    bool reached = (old_v < new_v) != (result < new_v);
    return reached ? new_v : result;
}

// uint_to_float_but_gradual.comp:29-39 (lower bound -inf, spread_kernel_width.cpp:25).
__global__ void k_kw_gradual(FluidBufs f, const uint32_t *ukw, const uint32_t *d_len, float speed) {
    const uint32_t n = d_len[kLenParticles];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float v = (float)ukw[i] * (1.0f / 262144.0f);
        v = move_towards_geo(f.kernel_width[i], v, speed);
        f.kernel_width[i] = fmaxf(v, __int_as_float(0xff800000));
    }
}

__global__ void k_pairs_total(const uint32_t *count, const uint32_t *d_len, unsigned long long *total) {
    const uint32_t n = d_len[kLenParticles];
    unsigned long long local = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) local += count[i];
    for (int off = 16; off > 0; off >>= 1) local += __shfl_down_sync(0xffffffffu, local, off);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(total, local);
}

}  // namespace

apbf_status update_transfers(apbf_ctx *ctx, cudaStream_t s) {
    const uint32_t cap = ctx->cfg.particle_capacity;
    const int g = grid_for(ctx, cap);
    FluidBufs &f = ctx->fl[ctx->fcur];
    const apbf_settings &st = ctx->settings;
    // k_fsm12 reads the old boundary distances and writes the new ones into the
    // spare array; the two arrays then swap (update_transfers.cpp:30,37)
    APBF_BEFORE_LAUNCH(ctx, s, "k_fsm12");
    k_fsm12<<<g, kBlock, 0, s>>>(f.pos, f.boundary_distance, ctx->old_bd, ctx->nearest, ctx->nb_count, ctx->nb_idx,
                                 ctx->row_stride, ctx->d_len);
    APBF_AFTER_LAUNCH(ctx, s, "k_fsm12");
    uint32_t *tmp = f.boundary_distance;
    f.boundary_distance = ctx->old_bd;
    ctx->old_bd = tmp;

    Fsm3Args a;
    a.f = f;
    a.nearest = ctx->nearest;
    a.pkind = ctx->proposal;
    a.psrc = ctx->list_a;
    a.ptgt = ctx->list_b;
    a.flag = ctx->flag_scan;
    a.d_len = ctx->d_len;
    a.split_c = (float)(cbrt(2.0) * 0.99);  // pow(2.0, 1.0 / DIMENSIONS) * 0.99 (find_split_and_merge_3.comp:90)
    a.sf = st.target_radius_scale_factor;
    a.rmin = st.smallest_target_radius;
    a.offset = st.target_radius_offset;
    a.merge = st.merge;
    a.split = st.split;
    a.update_target = st.update_target_radius;
    a.bd_mode = st.base_kernel_width_on_boundary_distance;
    APBF_BEFORE_LAUNCH(ctx, s, "k_fsm3");
    k_fsm3<<<g, kBlock, 0, s>>>(a);
    APBF_AFTER_LAUNCH(ctx, s, "k_fsm3");
    // proposals in index order
    APBF_CUDA(cudaMemcpyAsync(ctx->scan_tmp, ctx->flag_scan, (size_t)cap * 4, cudaMemcpyDeviceToDevice, s));
    apbf_status r = prefix_sum_device(ctx, ctx->scan_tmp, ctx->d_len + kLenParticles, cap, s);
    if (r != APBF_OK) return r;
    APBF_BEFORE_LAUNCH(ctx, s, "k_compact_ids");
    k_compact_ids<<<g, kBlock, 0, s>>>(ctx->flag_scan, ctx->scan_tmp, ctx->claim, ctx->d_len,
                                       ctx->d_len + kLenScratch);
    APBF_AFTER_LAUNCH(ctx, s, "k_compact_ids");

    ClaimArgs c;
    c.list = ctx->claim;
    c.count = ctx->d_len + kLenScratch;
    c.pkind = ctx->proposal;
    c.psrc = ctx->list_a;
    c.ptgt = ctx->list_b;
    c.owner = ctx->owner;
    c.state = ctx->decided;
    c.transferring = f.transferring;
    c.t = ctx->tr[ctx->tcur];
    c.d_len = ctx->d_len;
    c.splits = ctx->ukw;
    c.max_transfers = ctx->cfg.transfer_capacity;
    c.particle_cap = cap;
    c.merge_ttl = fmaxf(0.0001f, st.merge_duration);
    c.split_ttl = -st.split_duration;
    c.st = ctx->status;
    APBF_BEFORE_LAUNCH(ctx, s, "k_claims");
    k_claims<<<1, kClaimThreads, 0, s>>>(c);
    APBF_AFTER_LAUNCH(ctx, s, "k_claims");
    if (st.split) {
        APBF_BEFORE_LAUNCH(ctx, s, "k_split");
        k_split<<<g, kBlock, 0, s>>>(f, ctx->ukw, ctx->d_len);
        APBF_AFTER_LAUNCH(ctx, s, "k_split");
        APBF_BEFORE_LAUNCH(ctx, s, "k_split_len");
        k_split_len<<<1, 1, 0, s>>>(ctx->d_len);
        APBF_AFTER_LAUNCH(ctx, s, "k_split_len");
    }
    return APBF_OK;
}

apbf_status particle_transfer(apbf_ctx *ctx, float dt, cudaStream_t s) {
    const uint32_t cap = ctx->cfg.particle_capacity;
    const uint32_t tcap = ctx->cfg.transfer_capacity;
    FluidBufs &f = ctx->fl[ctx->fcur];
    TransferBufs &t = ctx->tr[ctx->tcur];
    uint32_t *pdel = ctx->flag_scan;   // per particle: deleted
    uint32_t *pscan = ctx->scan_tmp;   // per particle: inclusive scan of kept
    uint32_t *tkeep = ctx->t_keep;     // per transfer: kept
    uint32_t *tscan = ctx->t_scan;     // per transfer: inclusive scan of kept
    APBF_CUDA(cudaMemsetAsync(pdel, 0, (size_t)cap * 4, s));
    APBF_BEFORE_LAUNCH(ctx, s, "k_transfer");
    k_transfer<<<grid_for(ctx, tcap), kBlock, 0, s>>>(f, t, pdel, tkeep, ctx->d_len, dt);
    APBF_AFTER_LAUNCH(ctx, s, "k_transfer");
    APBF_BEFORE_LAUNCH(ctx, s, "k_transfer_keep2");
    k_transfer_keep2<<<grid_for(ctx, tcap), kBlock, 0, s>>>(t, tkeep, pdel, ctx->d_len);
    APBF_AFTER_LAUNCH(ctx, s, "k_transfer_keep2");
    APBF_BEFORE_LAUNCH(ctx, s, "k_keep_flags");
    k_keep_flags<<<grid_for(ctx, cap), kBlock, 0, s>>>(pdel, pscan, ctx->d_len);
    APBF_AFTER_LAUNCH(ctx, s, "k_keep_flags");
    apbf_status r = prefix_sum_device(ctx, pscan, ctx->d_len + kLenParticles, cap, s);
    if (r != APBF_OK) return r;
    APBF_CUDA(cudaMemcpyAsync(tscan, tkeep, (size_t)tcap * 4, cudaMemcpyDeviceToDevice, s));
    r = prefix_sum_device(ctx, tscan, ctx->d_len + kLenTransfers, tcap, s);
    if (r != APBF_OK) return r;
    FluidBufs &alt = ctx->fl[ctx->fcur ^ 1];
    TransferBufs &talt = ctx->tr[ctx->tcur ^ 1];
    APBF_BEFORE_LAUNCH(ctx, s, "k_compact_particles");
    k_compact_particles<<<grid_for(ctx, cap), kBlock, 0, s>>>(f, alt, pscan, pdel, ctx->d_len);
    APBF_AFTER_LAUNCH(ctx, s, "k_compact_particles");
    APBF_BEFORE_LAUNCH(ctx, s, "k_compact_transfers");
    k_compact_transfers<<<grid_for(ctx, tcap), kBlock, 0, s>>>(t, talt, tkeep, tscan, pscan, ctx->d_len);
    APBF_AFTER_LAUNCH(ctx, s, "k_compact_transfers");
    APBF_BEFORE_LAUNCH(ctx, s, "k_compact_lengths");
    k_compact_lengths<<<1, 1, 0, s>>>(pscan, tscan, ctx->d_len);
    APBF_AFTER_LAUNCH(ctx, s, "k_compact_lengths");
    ctx->fcur ^= 1;
    ctx->tcur ^= 1;
    return APBF_OK;
}

apbf_status spread_kernel_width(apbf_ctx *ctx, cudaStream_t s) {
    const uint32_t cap = ctx->cfg.particle_capacity;
    const int g = grid_for(ctx, cap);
    FluidBufs &f = ctx->fl[ctx->fcur];
    const int use_target = ctx->settings.base_kernel_width_on_target_radius;
    APBF_BEFORE_LAUNCH(ctx, s, "k_kw_init");
    k_kw_init<<<g, kBlock, 0, s>>>(f, ctx->ukw, ctx->d_len, use_target);
    APBF_AFTER_LAUNCH(ctx, s, "k_kw_init");
    APBF_BEFORE_LAUNCH(ctx, s, "k_kw_spread");
    k_kw_spread<<<g, kBlock, 0, s>>>(f, ctx->ukw, ctx->nb_count, ctx->nb_idx, ctx->row_stride, ctx->d_len, use_target);
    APBF_AFTER_LAUNCH(ctx, s, "k_kw_spread");
    APBF_BEFORE_LAUNCH(ctx, s, "k_kw_gradual");
    k_kw_gradual<<<g, kBlock, 0, s>>>(f, ctx->ukw, ctx->d_len, ctx->settings.kernel_width_adaption_speed);
    APBF_AFTER_LAUNCH(ctx, s, "k_kw_gradual");
    // the pruned rows: new pair count and transposed rows
    APBF_CUDA(cudaMemsetAsync(ctx->d_pairs, 0, sizeof(unsigned long long), s));
    APBF_BEFORE_LAUNCH(ctx, s, "k_pairs_total");
    k_pairs_total<<<g, kBlock, 0, s>>>(ctx->nb_count, ctx->d_len, ctx->d_pairs);
    APBF_AFTER_LAUNCH(ctx, s, "k_pairs_total");
    return build_reverse_rows(ctx, s);
}

}  // namespace apbf
