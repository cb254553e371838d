/*
 * apbf_oracle.c -- CPU restatement of the APBF substep shaders (TEST INFRASTRUCTURE).
 *
 * This is the correctness oracle for the CUDA implementation; the product never
 * links or calls it.  See apbf_oracle.h for the precision policy.  Build with
 * -ffp-contract=off so that the FP32-emulated stages round exactly like the
 * device code (which uses __fmul_rn / __fadd_rn where the order matters).
 *
 * Canonical rules (the reference is racy or undefined at these points; the
 * CUDA path implements the same rules):
 *  C1 cell of a position: clamp(floor((X - Xmin) * 2^L / (Xmax - Xmin)), 0, 2^L-1)
 *     on 2^18 fixed-point int64 (reference: FP32 uint() conversion,
 *     calculate_position_hash.comp:23-26, neighborhood_green.comp:35-37).
 *  C2 neighbour predicate: j != i and |X_j - X_i|^2 <= R_i^2 in exact integers,
 *     R_i = min(floor(kw_i * range_scale * 2^18), 2^31 - 1) evaluated in FP64 from
 *     the FP32 inputs (reference: FP32 distance(), neighborhood_green.comp:83).
 *  C3 sort: stable LSD by key from the identity permutation (test.cpp:335).
 *  C4 float -> int conversions truncate toward zero and saturate; NaN -> 0
 *     (GLSL int()/uint(); out-of-range is undefined in GLSL).
 *  C5 fixed-point lengths in split/merge: floor(isqrt(int64 |d|^2))
 *     (find_split_and_merge_1.comp:31, _2.comp:33 use FP32 length()).
 *  C6 nearest-neighbour tie: smallest j (find_split_and_merge_2.comp:35-37 is
 *     last-writer-wins); a particle without neighbours has no nearest neighbour
 *     and does not merge (the reference reads an uninitialised entry).
 *  C7 claims: sequential semantics in particle-index order
 *     (find_split_and_merge_3.comp:94-121 races on atomicExchange); capacity
 *     limits keep the first accepted transfers / splits in index order and
 *     release the rest for this substep.
 *  C8 append order of transfers, splits and list edits: index order.
 *  C9 a split duplicate has inverse mass +inf (initialize_split_particles.comp:31
 *     writes the undefined integer 1/0); particle_transfer then gives the target
 *     inverse mass invMassS / factor, the limit of invMassS*invMassT*normFactor
 *     (particle_transfer.comp:61 would produce inf*0 = NaN).
 *  C10 pow(x, 3) in the merge test is x*x*x in FP32.
 *  C11 the box-collision jitter uses the particle's sorted id
 *      (box_collision.comp:46 uses the racy order of the pool's index list).
 *  C12 quadratic-spike height uses (h - |r|)^2 for |r| < h (kernels.glsl:69
 *      raises a negative base to pow(), which GLSL leaves undefined).
 */
#include "apbf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define F32(x) ((double)(float)(x))
static const double kPi = F32(3.14159265);          /* kernels.glsl:1 */
static const double kTwoThirds = F32(2.0f / 3.0f);  /* 2.0f / DIMENSIONS */

/* The kernels and the incompressibility passes compute in or_real: double (the
 * oracle), or float in the FP32 build (-DOR_FP32) that is only timed as a CPU
 * baseline.  In the double build every macro below is the identity. */
#ifdef OR_FP32
#define RPOW powf
#define REXP expf
#define RSQRT sqrtf
#define RFMIN fminf
#else
#define RPOW pow
#define REXP exp
#define RSQRT sqrt
#define RFMIN fmin
#endif
#ifdef OR_FP32
typedef float or_real;
#else
typedef double or_real;
#endif
#define RL(x) ((or_real)(x))
#define F32R(x) ((or_real)(float)(x))
#define PI_R ((or_real)kPi)
#define TWO_THIRDS_R ((or_real)kTwoThirds)

/* ------------------------------------------------------------------ */
/* conversions (C4)                                                    */
/* ------------------------------------------------------------------ */
static int32_t f2i(double x) {
    if (x != x) return 0;
    if (x >= 2147483647.0) return INT32_MAX;
    if (x <= -2147483648.0) return INT32_MIN;
    return (int32_t)x; /* C truncates toward zero */
}
static uint32_t f2u(double x) {
    if (x != x || x <= 0.0) return 0u;
    if (x >= 4294967295.0) return UINT32_MAX;
    return (uint32_t)x;
}
static int32_t f2i_f(float x) { return f2i((double)x); }
static uint32_t f2u_f(float x) { return f2u((double)x); }
static int32_t wrap_add(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }

/* ------------------------------------------------------------------ */
/* primitives                                                          */
/* ------------------------------------------------------------------ */

/* Inclusive prefix sum (algorithms.cpp:93-118, prefix_sum_apply_on_block_level.comp). */
void or_prefix_sum_inclusive(const uint32_t *in, uint32_t *out, size_t n) {
    uint32_t s = 0;
    for (size_t i = 0; i < n; ++i) {
        s += in[i];
        out[i] = s;
    }
}

/* Stable key/value sort (algorithms.cpp:59-91): LSD passes of 8-bit digits. */
void or_sort_pairs_stable(const uint32_t *keys, const uint32_t *vals, size_t n, uint32_t *out_keys,
                          uint32_t *out_vals) {
    uint32_t *ka = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    uint32_t *va = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    uint32_t *kb = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    uint32_t *vb = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    memcpy(ka, keys, n * sizeof(uint32_t));
    memcpy(va, vals, n * sizeof(uint32_t));
    for (int shift = 0; shift < 32; shift += 8) {
        size_t count[257];
        memset(count, 0, sizeof(count));
        for (size_t i = 0; i < n; ++i) count[((ka[i] >> shift) & 255u) + 1]++;
        for (int d = 0; d < 256; ++d) count[d + 1] += count[d];
        for (size_t i = 0; i < n; ++i) {
            size_t p = count[(ka[i] >> shift) & 255u]++;
            kb[p] = ka[i];
            vb[p] = va[i];
        }
        uint32_t *t = ka; ka = kb; kb = t;
        t = va; va = vb; vb = t;
    }
    memcpy(out_keys, ka, n * sizeof(uint32_t));
    memcpy(out_vals, va, n * sizeof(uint32_t));
    free(ka); free(va); free(kb); free(vb);
}

/* gpu_list::apply_edit (gpu_list.h:125-135) via copy_scattered_read.comp:20-30. */
void or_apply_edit_u32(const uint32_t *src, const uint32_t *edit, size_t n_edit, uint32_t stride_words,
                       uint32_t *dst) {
    for (size_t e = 0; e < n_edit; ++e)
        for (uint32_t o = 0; o < stride_words; ++o) dst[e * stride_words + o] = src[(size_t)edit[e] * stride_words + o];
}

/* Edit list of indexed_list::delete_these (indexed_list.h:125-138): scattered_write
 * marks deleted hidden entries with 0, prefix_sum, find_value_changes.comp:15-28
 * emits the surviving hidden ids in increasing order.  Returns the new length. */
uint32_t or_delete_edit_list(uint32_t n_hidden, const uint32_t *deleted, uint32_t n_deleted, uint32_t *edit) {
    uint32_t *helper = (uint32_t *)calloc(n_hidden ? n_hidden : 1, sizeof(uint32_t));
    for (uint32_t i = 0; i < n_hidden; ++i) helper[i] = 1u;
    for (uint32_t k = 0; k < n_deleted; ++k) helper[deleted[k]] = 0u;
    or_prefix_sum_inclusive(helper, helper, n_hidden);
    uint32_t len = 0;
    for (uint32_t id = 0; id < n_hidden; ++id) {
        uint32_t cur = helper[id];
        uint32_t prev = id == 0 ? 0u : helper[id - 1];
        if (id == n_hidden - 1) len = cur;
        if (cur != prev) edit[prev] = id;
    }
    free(helper);
    return len;
}

/* indexed_list::apply_hidden_edit (indexed_list.h:288-308): after the hidden list
 * is rebuilt from `edit` (new hidden id e takes old hidden id edit[e]), an index
 * list pointing into the hidden list gets one entry e for every old entry equal
 * to edit[e].  atomic_swap.comp chains equal entries and
 * generate_new_index_and_edit_list.comp emits them with an atomic counter; the
 * canonical order is by e, then by old position (C8).  new_edit (may be NULL)
 * receives, per new entry, the old index-list position it came from.  Returns
 * the new length (at most max_out). */
uint32_t or_remap_index_list(const uint32_t *list, uint32_t n_list, const uint32_t *edit, uint32_t n_edit,
                             uint32_t n_hidden_old, uint32_t *out, uint32_t *new_edit, uint32_t max_out) {
    uint32_t *head = (uint32_t *)malloc((size_t)(n_hidden_old ? n_hidden_old : 1) * sizeof(uint32_t));
    uint32_t *next = (uint32_t *)malloc((size_t)(n_list ? n_list : 1) * sizeof(uint32_t));
    for (uint32_t h = 0; h < n_hidden_old; ++h) head[h] = UINT32_MAX;
    for (uint32_t p = n_list; p-- > 0;) { /* build chains in increasing position order */
        uint32_t h = list[p];
        if (h >= n_hidden_old) continue;
        next[p] = head[h];
        head[h] = p;
    }
    uint32_t m = 0;
    for (uint32_t e = 0; e < n_edit; ++e) {
        uint32_t h = edit[e];
        if (h >= n_hidden_old) continue;
        for (uint32_t p = head[h]; p != UINT32_MAX; p = next[p]) {
            if (m >= max_out) break;
            out[m] = e;
            if (new_edit) new_edit[m] = p;
            ++m;
        }
    }
    free(head);
    free(next);
    return m;
}

/* ------------------------------------------------------------------ */
/* neighbour search                                                    */
/* ------------------------------------------------------------------ */

void or_fixed_bounds(const float minp[3], const float maxp[3], int64_t out_min[3], int64_t out_max[3]) {
    for (int d = 0; d < 3; ++d) {
        out_min[d] = (int64_t)llround((double)minp[d] * OR_POS_RESOLUTION);
        out_max[d] = (int64_t)llround((double)maxp[d] * OR_POS_RESOLUTION);
        if (out_max[d] <= out_min[d]) out_max[d] = out_min[d] + 1;
    }
}

/* C1: cell coordinate of a fixed-point coordinate. */
uint32_t or_cell_coord(int64_t x, int64_t xmin, int64_t xmax, uint32_t log2res) {
    const int64_t cells = (int64_t)1 << log2res;
    if (x <= xmin) return 0u;
    if (x >= xmax) return (uint32_t)(cells - 1);
    int64_t c = ((x - xmin) << log2res) / (xmax - xmin);
    if (c > cells - 1) c = cells - 1;
    return (uint32_t)c;
}

/* Z-order interleave, bit i of dimension d -> bit i*3+d (calculate_position_hash.comp:29-36). */
uint32_t or_morton(const uint32_t c[3], uint32_t log2res) {
    uint32_t r = 0u;
    for (uint32_t i = 0; i < log2res; ++i)
        for (uint32_t d = 0; d < 3; ++d) r += ((c[d] >> i) & 1u) << (i * 3u + d);
    return r;
}

/* calculate_position_hash.comp:39-46 */
void or_position_keys(const int32_t *pos4, size_t n, const float minp[3], const float maxp[3],
                      uint32_t log2res, uint32_t *keys) {
    int64_t lo[3], hi[3];
    or_fixed_bounds(minp, maxp, lo, hi);
    for (size_t i = 0; i < n; ++i) {
        uint32_t c[3];
        for (int d = 0; d < 3; ++d) c[d] = or_cell_coord(pos4[4 * i + d], lo[d], hi[d], log2res);
        keys[i] = or_morton(c, log2res);
    }
}

/* find_value_ranges.comp:15-31 with the zero fill of neighborhood_green.cpp:61-62. */
void or_cell_ranges(const uint32_t *sorted_keys, size_t n, uint32_t ncells, uint32_t *start, uint32_t *end) {
    memset(start, 0, (size_t)ncells * sizeof(uint32_t));
    memset(end, 0, (size_t)ncells * sizeof(uint32_t));
    for (size_t id = 0; id < n; ++id) {
        uint32_t cur = sorted_keys[id];
        uint32_t prev = id == 0 ? cur : sorted_keys[id - 1];
        if (id == 0 || cur != prev) start[cur] = (uint32_t)id;
        if (id != 0 && cur != prev) end[prev] = (uint32_t)id;
        if (id == n - 1) end[cur] = (uint32_t)id + 1u;
    }
}

/* C2: fixed-point search radius. */
int64_t or_range_fixed(float kernel_width, float range_scale) {
    double r = (double)kernel_width * (double)range_scale * OR_POS_RESOLUTION;
    if (!(r >= 0.0)) return -1;
    if (r > 2147483647.0) r = 2147483647.0; /* positions are int32: no distance needs more */
    return (int64_t)floor(r);
}

static int within(const int32_t *a, const int32_t *b, int64_t R) {
    if (R < 0) return 0;
    uint64_t s = 0;
    for (int d = 0; d < 3; ++d) {
        int64_t dd = (int64_t)b[d] - (int64_t)a[d];
        if (dd < 0) dd = -dd;
        if (dd > R) return 0;
        s += (uint64_t)(dd * dd);
    }
    return s <= (uint64_t)R * (uint64_t)R;
}

static int cmp_u32(const void *a, const void *b) {
    uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
    return x < y ? -1 : x > y;
}

/* neighborhood_green.comp:49-87: walk the cells overlapping [X - R, X + R]. */
uint64_t or_neighbors_build(const int32_t *pos4, const float *range, float range_scale, size_t n,
                            const float minp[3], const float maxp[3], uint32_t log2res,
                            const uint32_t *cell_start, const uint32_t *cell_end, or_neighbors *nb) {
    int64_t lo[3], hi[3];
    or_fixed_bounds(minp, maxp, lo, hi);
    uint64_t total = 0;
    int write = 1;
    nb->n = (uint32_t)n;
    nb->offsets[0] = 0;
    for (size_t i = 0; i < n; ++i) {
        const int32_t *p = pos4 + 4 * i;
        int64_t R = or_range_fixed(range[i], range_scale);
        uint64_t row_begin = total;
        if (R >= 0) {
            uint32_t cmin[3], cmax[3];
            for (int d = 0; d < 3; ++d) {
                cmin[d] = or_cell_coord((int64_t)p[d] - R, lo[d], hi[d], log2res);
                cmax[d] = or_cell_coord((int64_t)p[d] + R, lo[d], hi[d], log2res);
            }
            uint32_t c[3];
            for (c[2] = cmin[2]; c[2] <= cmax[2]; ++c[2])
                for (c[1] = cmin[1]; c[1] <= cmax[1]; ++c[1])
                    for (c[0] = cmin[0]; c[0] <= cmax[0]; ++c[0]) {
                        uint32_t key = or_morton(c, log2res);
                        for (uint32_t j = cell_start[key]; j < cell_end[key]; ++j) {
                            if (j == i) continue;
                            if (!within(p, pos4 + 4 * (size_t)j, R)) continue;
                            if (total >= nb->cap) write = 0;
                            if (write) nb->idx[total] = j;
                            ++total;
                        }
                    }
        }
        if (write) {
            qsort(nb->idx + row_begin, (size_t)(total - row_begin), sizeof(uint32_t), cmp_u32);
            nb->offsets[i + 1] = (uint32_t)total;
        }
    }
    return total;
}

/* O(n^2) version of the same predicate, for tiny self-checks. */
uint64_t or_neighbors_brute(const int32_t *pos4, const float *range, float range_scale, size_t n,
                            or_neighbors *nb) {
    uint64_t total = 0;
    int write = 1;
    nb->n = (uint32_t)n;
    nb->offsets[0] = 0;
    for (size_t i = 0; i < n; ++i) {
        int64_t R = or_range_fixed(range[i], range_scale);
        for (size_t j = 0; j < n; ++j) {
            if (j == i || !within(pos4 + 4 * i, pos4 + 4 * j, R)) continue;
            if (total >= nb->cap) write = 0;
            if (write) nb->idx[total] = (uint32_t)j;
            ++total;
        }
        if (write) nb->offsets[i + 1] = (uint32_t)total;
    }
    return total;
}

static void permute_f(float *a, const uint32_t *perm, size_t n, size_t w, void *tmp) {
    float *t = (float *)tmp;
    for (size_t k = 0; k < n; ++k) memcpy(t + k * w, a + (size_t)perm[k] * w, w * sizeof(float));
    memcpy(a, t, n * w * sizeof(float));
}
static void permute_u(uint32_t *a, const uint32_t *perm, size_t n, size_t w, void *tmp) {
    uint32_t *t = (uint32_t *)tmp;
    for (size_t k = 0; k < n; ++k) memcpy(t + k * w, a + (size_t)perm[k] * w, w * sizeof(uint32_t));
    memcpy(a, t, n * w * sizeof(uint32_t));
}

/* Gather every attribute by an edit list (new id -> old id), gpu_list.h:125-135. */
static void fluid_apply_edit(or_fluid *f, const uint32_t *edit, uint32_t n_new) {
    size_t m = n_new > f->n ? n_new : f->n;
    void *tmp = malloc((m ? m : 1) * 16);
    permute_u((uint32_t *)f->pos, edit, n_new, 4, tmp);
    permute_f(f->vel, edit, n_new, 4, tmp);
    permute_f(f->inv_mass, edit, n_new, 1, tmp);
    permute_f(f->radius, edit, n_new, 1, tmp);
    permute_u((uint32_t *)f->pos_backup, edit, n_new, 4, tmp);
    permute_u(f->transferring, edit, n_new, 1, tmp);
    permute_f(f->target_radius, edit, n_new, 1, tmp);
    permute_f(f->kernel_width, edit, n_new, 1, tmp);
    permute_f(f->boundariness, edit, n_new, 1, tmp);
    permute_u(f->boundary_distance, edit, n_new, 1, tmp);
    f->n = n_new;
    free(tmp);
}

/* Remap transfer particle ids after a particle edit (indexed_list.h:288-308):
 * a transfer survives iff both of its particles survive; order is kept (C8). */
static void transfers_remap(or_transfers *t, const uint32_t *edit, uint32_t n_new, uint32_t n_old) {
    if (!t || t->n == 0) return;
    uint32_t *inv = (uint32_t *)malloc((n_old ? n_old : 1) * sizeof(uint32_t));
    for (uint32_t i = 0; i < n_old; ++i) inv[i] = UINT32_MAX;
    for (uint32_t k = 0; k < n_new; ++k)
        if (inv[edit[k]] == UINT32_MAX) inv[edit[k]] = k;
    uint32_t m = 0;
    for (uint32_t k = 0; k < t->n; ++k) {
        uint32_t s = t->source[k] < n_old ? inv[t->source[k]] : UINT32_MAX;
        uint32_t g = t->target[k] < n_old ? inv[t->target[k]] : UINT32_MAX;
        if (s == UINT32_MAX || g == UINT32_MAX) continue;
        t->source[m] = s;
        t->target[m] = g;
        t->time_left[m] = t->time_left[k];
        ++m;
    }
    t->n = m;
    free(inv);
}

/* neighborhood_green::apply (neighborhood_green.cpp:27-77). */
uint64_t or_neighborhood_green(or_fluid *f, or_transfers *t, float range_scale, const float minp[3],
                               const float maxp[3], uint32_t log2res, or_neighbors *nb,
                               uint32_t *perm_out, uint32_t *keys_out) {
    size_t n = f->n;
    uint32_t ncells = 1u << (3u * log2res);
    uint32_t *keys = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    uint32_t *seq = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    uint32_t *skeys = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    uint32_t *perm = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    uint32_t *cs = (uint32_t *)malloc((size_t)ncells * sizeof(uint32_t));
    uint32_t *ce = (uint32_t *)malloc((size_t)ncells * sizeof(uint32_t));
    or_position_keys(f->pos, n, minp, maxp, log2res, keys);
    for (size_t i = 0; i < n; ++i) seq[i] = (uint32_t)i;
    or_sort_pairs_stable(keys, seq, n, skeys, perm);
    fluid_apply_edit(f, perm, (uint32_t)n);
    transfers_remap(t, perm, (uint32_t)n, (uint32_t)n);
    or_cell_ranges(skeys, n, ncells, cs, ce);
    uint64_t total = or_neighbors_build(f->pos, f->kernel_width, range_scale, n, minp, maxp, log2res, cs, ce, nb);
    if (perm_out) memcpy(perm_out, perm, n * sizeof(uint32_t));
    if (keys_out) memcpy(keys_out, skeys, n * sizeof(uint32_t));
    free(keys); free(seq); free(skeys); free(perm); free(cs); free(ce);
    return total;
}

/* ------------------------------------------------------------------ */
/* neighborhood_binary_search (neighborhood_binary_search.cpp:22-75)  */
/* ------------------------------------------------------------------ */
/* calculate_position_code.comp:22-62: code bit 3b + a is bit b of axis a, the
 * coordinates taken as uint32; out[0] holds code bits 0-31, out[2] bits 64-95. */
void or_position_code96(const int32_t *p, uint32_t out[3]) {
    out[0] = out[1] = out[2] = 0;
    for (uint32_t b = 0; b < 32; ++b)
        for (uint32_t a = 0; a < 3; ++a) {
            uint32_t bit = 3u * b + a;
            if (((uint32_t)p[a] >> b) & 1u) out[bit / 32u] |= 1u << (bit % 32u);
        }
}

static int cmp96(const uint32_t *a, const uint32_t *b) {
    for (int w = 2; w >= 0; --w)
        if (a[w] != b[w]) return a[w] < b[w] ? -1 : 1;
    return 0;
}

/* neighborhood_binary_search.comp:186-275 with the canonical rules: level k the
 * smallest with 2^k >= R; cells visited in the shader's order (x fastest, offsets
 * -1, 0, +1; at k = 31 the offset +1 equals -1 and is skipped); each cell is the run
 * of sorted codes in [corner code, corner code | low 3k bits]; exact predicate. */
uint64_t or_neighbors_binary_search(const int32_t *pos4, const uint32_t *codes3, const float *range,
                                    float range_scale, size_t n, or_neighbors *nb) {
    uint64_t total = 0;
    int write = 1;
    nb->n = (uint32_t)n;
    nb->offsets[0] = 0;
    for (size_t i = 0; i < n; ++i) {
        const int32_t *p = pos4 + 4 * i;
        int64_t R = or_range_fixed(range[i], range_scale);
        if (R >= 0) {
            uint32_t k = 0;
            while (((uint64_t)1 << k) < (uint64_t)R) ++k;
            uint32_t nd = k == 31 ? 2u : 3u;
            for (uint32_t dz = 0; dz < nd; ++dz)
                for (uint32_t dy = 0; dy < nd; ++dy)
                    for (uint32_t dx = 0; dx < nd; ++dx) {
                        uint32_t d[3] = {dx, dy, dz};
                        int32_t corner[3], top[3];
                        for (int a = 0; a < 3; ++a) {
                            uint64_t c = (((uint64_t)((uint32_t)p[a] >> k) + d[a] + 0xffffffffull) << k) & 0xffffffffull;
                            uint64_t low = k ? (((uint64_t)1 << k) - 1) : 0;
                            corner[a] = (int32_t)(uint32_t)c;
                            top[a] = (int32_t)(uint32_t)(c | low);
                        }
                        uint32_t first[3], last[3];
                        or_position_code96(corner, first);
                        or_position_code96(top, last);
                        /* lower bound: first j with code >= first */
                        size_t lo = 0, hi = n;
                        while (lo < hi) {
                            size_t mid = (lo + hi) / 2;
                            if (cmp96(codes3 + 3 * mid, first) < 0) lo = mid + 1; else hi = mid;
                        }
                        for (size_t j = lo; j < n && cmp96(codes3 + 3 * j, last) <= 0; ++j) {
                            if (j == i || !within(p, pos4 + 4 * j, R)) continue;
                            if (total >= nb->cap) write = 0;
                            if (write) nb->idx[total] = (uint32_t)j;
                            ++total;
                        }
                    }
        }
        if (write) nb->offsets[i + 1] = (uint32_t)total;
    }
    return total;
}

/* neighborhood_binary_search::apply: codes, stable sort by the 96-bit code (three
 * stable passes, least significant word first), reorder, codes of the sorted list,
 * rows.  perm_out / codes_out (may be NULL) receive the permutation and the sorted
 * codes (3 words per particle). */
uint64_t or_neighborhood_binary_search(or_fluid *f, or_transfers *t, float range_scale, or_neighbors *nb,
                                       uint32_t *perm_out, uint32_t *codes_out) {
    size_t n = f->n, m = n ? n : 1;
    uint32_t *codes = (uint32_t *)malloc(m * 3 * sizeof(uint32_t));
    uint32_t *keys = (uint32_t *)malloc(m * sizeof(uint32_t));
    uint32_t *vals = (uint32_t *)malloc(m * sizeof(uint32_t));
    uint32_t *skeys = (uint32_t *)malloc(m * sizeof(uint32_t));
    uint32_t *perm = (uint32_t *)malloc(m * sizeof(uint32_t));
    for (size_t i = 0; i < n; ++i) {
        or_position_code96(f->pos + 4 * i, codes + 3 * i);
        perm[i] = (uint32_t)i;
    }
    for (int w = 0; w < 3; ++w) {
        for (size_t k = 0; k < n; ++k) {
            keys[k] = codes[3 * (size_t)perm[k] + (size_t)w];
            vals[k] = perm[k];
        }
        or_sort_pairs_stable(keys, vals, n, skeys, perm);
    }
    fluid_apply_edit(f, perm, (uint32_t)n);
    transfers_remap(t, perm, (uint32_t)n, (uint32_t)n);
    for (size_t i = 0; i < n; ++i) or_position_code96(f->pos + 4 * i, codes + 3 * i);
    uint64_t total = or_neighbors_binary_search(f->pos, codes, f->kernel_width, range_scale, n, nb);
    if (perm_out) memcpy(perm_out, perm, n * sizeof(uint32_t));
    if (codes_out) memcpy(codes_out, codes, n * 3 * sizeof(uint32_t));
    free(codes); free(keys); free(vals); free(skeys); free(perm);
    return total;
}

/* ------------------------------------------------------------------ */
/* smoothing kernels (kernels.glsl), in or_real (FP64; FP32 build)   */
/* ------------------------------------------------------------------ */
static or_real dot3(const or_real a[3], const or_real b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static or_real len3(const or_real a[3]) { return RSQRT(dot3(a, a)); }

static or_real gauss_height_param(or_real kw) {  /* kernels.glsl:104 */
    or_real half = kw / RL(2.0);
    return F32R(0.6f) / (half * half * half);
}
static or_real gauss_height(const or_real r[3], or_real height) {  /* kernels.glsl:84-89 */
    or_real ivw = RPOW(height, TWO_THIRDS_R);
    or_real ivd = ivw * PI_R;
    return REXP(-dot3(r, r) * ivd) * RPOW(ivw, RL(1.5));
}

static or_real kheight(int id, const or_real r[3], or_real h) {
    or_real dist = len3(r);
    switch (id) {
    case 0: { /* cubic, kernels.glsl:18-31 */
        if (dist > h) return RL(0.0);
        or_real q = dist / h;
        or_real k = RL(8.0) / (PI_R * h * h * h);
        if (q <= RL(0.5)) return k * (RL(6.0) * q * q * q - RL(6.0) * q * q + RL(1.0));
        return k * (RL(2.0) * RPOW(RL(1.0) - q, RL(3.0)));
    }
    case 1: return gauss_height(r, gauss_height_param(h));
    case 2: { /* poly6, kernels.glsl:3-9 */
        or_real r2 = dot3(r, r), h2 = h * h;
        if (r2 > h2) return RL(0.0);
        return RL(315.0) * RPOW(h2 - r2, RL(3.0)) / (RL(64.0) * PI_R * RPOW(h, RL(9.0)));
    }
    case 3: { /* cone, kernels.glsl:48-52 */
        or_real height = RL(3.0) / (PI_R * RPOW(h, RL(3.0)));
        or_real v = (RL(1.0) - dist / h) * height;
        return v > RL(0.0) ? v : RL(0.0);
    }
    case 4: { /* quadratic spike, kernels.glsl:62-70 (C12) */
        or_real a = RL(15.0) / (RL(2.0) * PI_R * RPOW(h, RL(5.0)));
        if (dist >= h) return RL(0.0);
        return a * (h - dist) * (h - dist);
    }
    default: return RL(0.0);
    }
}

static void kgrad(int id, const or_real r[3], or_real h, or_real out[3]) {
    or_real dist = len3(r);
    out[0] = out[1] = out[2] = RL(0.0);
    switch (id) {
    case 0: { /* kernels.glsl:33-46 */
        if (dist > h || dist < F32R(0.0001f)) return;
        or_real q = dist / h;
        or_real l = RL(48.0) / (PI_R * h * h * h);
        or_real s = q <= RL(0.5) ? l * q * (RL(3.0) * q - RL(2.0)) : l * (-(RL(1.0) - q) * (RL(1.0) - q));
        or_real inv = RL(1.0) / (dist * h);
        for (int d = 0; d < 3; ++d) out[d] = s * (r[d] * inv);
        return;
    }
    case 1: { /* kernels.glsl:91-97 */
        if (dist < F32R(0.0001f)) return;
        or_real height = gauss_height_param(h);
        or_real ivd = RPOW(height, TWO_THIRDS_R) * PI_R;
        or_real s = -gauss_height(r, height) * RL(2.0) * dist * ivd;
        for (int d = 0; d < 3; ++d) out[d] = s * (r[d] / dist);
        return;
    }
    case 2: { /* spiky, kernels.glsl:11-16 */
        if (dist > h || dist < F32R(0.0001f)) return;
        or_real s = -RL(45.0) * (h - dist) * (h - dist) / (PI_R * RPOW(h, RL(6.0)));
        for (int d = 0; d < 3; ++d) out[d] = s * (r[d] / dist);
        return;
    }
    case 3: { /* cone, kernels.glsl:54-60 */
        or_real st = RL(3.0) / (PI_R * RPOW(h, RL(4.0)));
        if (dist > h || dist < F32R(0.0001f)) return;
        for (int d = 0; d < 3; ++d) out[d] = -r[d] * (st / dist);
        return;
    }
    case 4: { /* kernels.glsl:72-82 */
        if (dist > h || dist < F32R(0.0001f)) return;
        or_real a = RL(15.0) / (RL(2.0) * PI_R * RPOW(h, RL(5.0)));
        or_real m = h - dist;
        if (m < RL(0.0)) m = RL(0.0);
        or_real s = -RL(2.0) * a * m / dist;
        for (int d = 0; d < 3; ++d) out[d] = s * r[d];
        return;
    }
    default: return;
    }
}

double or_kernel_height(int id, const double r[3], double h) {
    const or_real rr[3] = {(or_real)r[0], (or_real)r[1], (or_real)r[2]};
    return (double)kheight(id, rr, (or_real)h);
}

void or_kernel_gradient(int id, const double r[3], double h, double out[3]) {
    const or_real rr[3] = {(or_real)r[0], (or_real)r[1], (or_real)r[2]};
    or_real o[3];
    kgrad(id, rr, (or_real)h, o);
    for (int d = 0; d < 3; ++d) out[d] = (double)o[d];
}

/* ------------------------------------------------------------------ */
/* incompressibility (incompressibility.cpp:12-45), in or_real        */
/* ------------------------------------------------------------------ */
static or_real move_towards_lin(or_real old_v, or_real new_v, or_real step) {  /* incompressibility_2.comp:37-41 */
    or_real s = new_v - old_v;
    if (s < -step) s = -step;
    if (s > step) s = step;
    return old_v + s;
}

void or_incompressibility_apply(or_fluid *f, const or_neighbors *nb, const or_settings *s, or_incomp_out *out) {
    const uint32_t n = f->n;
    uint32_t *dens = (uint32_t *)calloc(n ? n : 1, sizeof(uint32_t));
    int32_t *gsum = (int32_t *)calloc(3 * (size_t)(n ? n : 1), sizeof(int32_t));
    uint32_t *sq = (uint32_t *)calloc(n ? n : 1, sizeof(uint32_t));
    int32_t *com = (int32_t *)calloc(4 * (size_t)(n ? n : 1), sizeof(int32_t));
    or_real *lambda = (or_real *)calloc(n ? n : 1, sizeof(or_real));
    or_real *div = (or_real *)calloc(n ? n : 1, sizeof(or_real));
    int32_t *shift = (int32_t *)calloc(3 * (size_t)(n ? n : 1), sizeof(int32_t));
    const or_real R = OR_POS_RESOLUTION;

    /* incompressibility_0.comp:32-45 */
    for (uint32_t i = 0; i < n; ++i) {
        or_real zero[3] = {0, 0, 0};
        dens[i] = f2u(kheight(s->height_kernel_id, zero, f->kernel_width[i]) / f->inv_mass[i] * R);
    }
    /* incompressibility_1.comp:37-69 (gather over row i; integer sums are order-free) */
    for (uint32_t i = 0; i < n; ++i) {
        const int32_t *p = f->pos + 4 * (size_t)i;
        or_real kw = f->kernel_width[i];
        for (uint32_t e = nb->offsets[i]; e < nb->offsets[i + 1]; ++e) {
            uint32_t j = nb->idx[e];
            const int32_t *q = f->pos + 4 * (size_t)j;
            or_real imn = f->inv_mass[j];
            or_real d[3], g[3];
            for (int c = 0; c < 3; ++c) d[c] = (or_real)(int32_t)((uint32_t)q[c] - (uint32_t)p[c]) / R;
            kgrad(s->gradient_kernel_id, d, kw, g);
            dens[i] += f2u(kheight(s->height_kernel_id, d, kw) / imn * R);
            for (int c = 0; c < 3; ++c) gsum[3 * i + c] = wrap_add(gsum[3 * i + c], f2i(g[c] / imn * R));
            sq[i] += f2u(dot3(g, g) / imn * R);
            for (int c = 0; c < 3; ++c) div[i] += ((or_real)f->vel[4 * (size_t)j + c] - f->vel[4 * (size_t)i + c]) * g[c] / imn;
            if (s->boundariness_calculation_method == 1) {
                for (int c = 0; c < 3; ++c)
                    com[4 * i + c] = wrap_add(com[4 * i + c],
                                              f2i((or_real)(int32_t)((uint32_t)q[c] - (uint32_t)p[c]) / (imn * kw)));
                com[4 * i + 3] = wrap_add(com[4 * i + 3], f2i(R / imn));
            }
        }
    }
    /* incompressibility_2.comp:71-110 */
    for (uint32_t i = 0; i < n; ++i) {
        or_real radius = f->radius[i], im = f->inv_mass[i], kw = f->kernel_width[i];
        or_real ird = RPOW(RL(2.0) * radius, RL(3.0)) * im;
        or_real density = (or_real)dens[i] / R;
        or_real wgs[3] = {(or_real)gsum[3 * i] / R, (or_real)gsum[3 * i + 1] / R, (or_real)gsum[3 * i + 2] / R};
        or_real sqs = (or_real)sq[i] / R;
        or_real wgsq = dot3(wgs, wgs);
        or_real sgl = RSQRT(wgsq) * ird;
        sqs += wgsq * im;
        or_real under = RL(1.0) - density * ird;
        if (s->update_boundariness) {
            or_real b;
            if (s->boundariness_calculation_method == 1) {
                or_real tm = (or_real)com[4 * i + 3] / R + RL(1.0) / im;
                or_real cv[3] = {(or_real)com[4 * i], (or_real)com[4 * i + 1], (or_real)com[4 * i + 2]};
                b = len3(cv) / (R * tm) * (or_real)s->boundariness_self_grad_length_factor;
            } else {
                or_real up = under > RL(0.0) ? under : RL(0.0);
                b = sgl * kw * (or_real)s->boundariness_self_grad_length_factor +
                    up * (or_real)s->boundariness_underpressure_factor;
            }
            b = b >= RL(1.0) ? RL(1.0) : RL(0.0);
            b = move_towards_lin((or_real)f->boundariness[i], b, (or_real)s->boundariness_adaption_speed);
            f->boundariness[i] = (float)(b < RL(1.0) ? b : RL(1.0));
        }
        or_real lam = under / (ird * ird * (sqs + F32R(0.01f)));
        or_real rmin2 = RL(2.0) * (or_real)s->smallest_target_radius;
        lam /= (rmin2 * rmin2 * rmin2) / ird * im;
        /* the applied lambda: pushes only (incompressibility_2.comp:106) */
        or_real applied = lam < RL(0.0) ? lam : RL(0.0);
        if (out && out->lambda_in) {
            if (out->lambda) out->lambda[i] = (float)lam;  /* the computed one, before the override */
            applied = (or_real)out->lambda_in[i];
        } else if (out && out->projected_acc && lam > RL(0.0)) {
            or_real a = RFMIN(lam, -(or_real)out->projected_acc[i]);
            applied = a > RL(0.0) ? a : RL(0.0);
        }
        if (out && out->lambda && !out->lambda_in) out->lambda[i] = (float)lam;
        if (out && out->applied) out->applied[i] = (float)applied;
        lambda[i] = applied;
        if (applied != RL(0.0)) {
            for (int c = 0; c < 3; ++c) shift[3 * i + c] = wrap_add(shift[3 * i + c], f2i(-wgs[c] * ird * (applied * im * R)));
        }
    }
    /* incompressibility_3.comp:48-67 */
    for (uint32_t i = 0; i < n; ++i) {
        const int32_t *p = f->pos + 4 * (size_t)i;
        or_real kw = f->kernel_width[i];
        or_real gi[3] = {(or_real)gsum[3 * i], (or_real)gsum[3 * i + 1], (or_real)gsum[3 * i + 2]};
        or_real gl = len3(gi);
        for (uint32_t e = nb->offsets[i]; e < nb->offsets[i + 1]; ++e) {
            uint32_t j = nb->idx[e];
            const int32_t *q = f->pos + 4 * (size_t)j;
            or_real d[3], g[3];
            for (int c = 0; c < 3; ++c) d[c] = (or_real)(int32_t)((uint32_t)q[c] - (uint32_t)p[c]) / R;
            kgrad(s->gradient_kernel_id, d, kw, g);
            if (s->boundariness_calculation_method == 2) {
                or_real l = len3(g);
                if (gl > RL(0.0) && l > RL(0.0)) {
                    or_real dd = RL(0.0);
                    for (int c = 0; c < 3; ++c) dd += (-gi[c] / gl) * (g[c] / l);
                    if (dd > F32R(0.6f)) f->boundariness[i] = 0.0f;
                }
            }
            if (lambda[i] == RL(0.0)) continue;
            for (int c = 0; c < 3; ++c) shift[3 * j + c] = wrap_add(shift[3 * j + c], f2i(g[c] * (lambda[i] * R)));
        }
    }
    for (uint32_t i = 0; i < n; ++i)
        for (int c = 0; c < 3; ++c) f->pos[4 * i + c] = wrap_add(f->pos[4 * i + c], shift[3 * i + c]);
    if (out) {
        if (out->density) memcpy(out->density, dens, n * sizeof(uint32_t));
        if (out->grad_sum) memcpy(out->grad_sum, gsum, 3 * (size_t)n * sizeof(int32_t));
        if (out->sq_grad_sum) memcpy(out->sq_grad_sum, sq, n * sizeof(uint32_t));
        if (out->divergence)
            for (uint32_t i = 0; i < n; ++i) out->divergence[i] = (float)div[i];
    }
    free(dens); free(gsum); free(sq); free(com); free(lambda); free(shift); free(div);
}

/* ------------------------------------------------------------------ */
/* substep glue, exact FP32                                            */
/* ------------------------------------------------------------------ */
static float fractf(float x) { return x - floorf(x); }

/* box_collision.comp:20-25 (hash31, MIT-licensed shadertoy hash, restated). */
static void hash31(float p, float out[3]) {
    float p3[3] = {fractf(p * 0.1031f), fractf(p * 0.1030f), fractf(p * 0.0973f)};
    float t = p3[0] * (p3[1] + 33.33f);
    t = t + p3[1] * (p3[2] + 33.33f);
    t = t + p3[2] * (p3[0] + 33.33f);
    p3[0] += t; p3[1] += t; p3[2] += t;
    out[0] = fractf((p3[0] + p3[1]) * p3[2]);
    out[1] = fractf((p3[0] + p3[2]) * p3[1]);
    out[2] = fractf((p3[1] + p3[2]) * p3[0]);
}

static void smallest_component(const float v[3], float m[3]) {  /* box_collision.comp:27-33 */
    int b1 = v[0] <= v[1], b2 = v[0] <= v[2], b3 = v[1] <= v[2];
    m[0] = (b1 && b2) ? 1.0f : 0.0f;
    m[1] = (!b1 && b3) ? 1.0f : 0.0f;
    m[2] = (!b2 && !b3) ? 1.0f : 0.0f;
}

/* box_collision.comp:35-60 */
/* box_collision.comp:35-57 for one box in its own frame (q relative to the frame,
 * box [lo, hi]); returns whether the particle moved. */
static int push_out(float q[3], const float lo[3], const float hi[3], float radius, const float h1[3],
                    const float h2[3]) {
    float tmin[3], tmax[3], m1[3], m2[3], neg[3];
    for (int c = 0; c < 3; ++c) {
        float bmin = (lo[c] - radius) - h1[c] * 0.05f;
        float bmax = (hi[c] + radius) + h2[c] * 0.05f;
        tmin[c] = bmin - q[c];
        tmax[c] = bmax - q[c];
        neg[c] = -tmin[c];
    }
    smallest_component(neg, m1);
    smallest_component(tmax, m2);
    for (int c = 0; c < 3; ++c) {
        tmin[c] *= m1[c];
        tmax[c] *= m2[c];
    }
    float dmin = -((tmin[0] + tmin[1]) + tmin[2]);
    float dmax = (tmax[0] + tmax[1]) + tmax[2];
    if (dmin <= 0.0f || dmax <= 0.0f) return 0;
    for (int c = 0; c < 3; ++c) q[c] += dmin < dmax ? tmin[c] : tmax[c];
    return 1;
}

void or_box_collision(or_fluid *f, const or_boxes *b) {
    for (uint32_t id = 0; id < f->n; ++id) {
        int32_t *ip = f->pos + 4 * (size_t)id;
        float pos[3] = {(float)ip[0] / 262144.0f, (float)ip[1] / 262144.0f, (float)ip[2] / 262144.0f};
        float radius = f->radius[id];
        for (uint32_t k = 0; k < b->n; ++k) {
            float h1[3], h2[3];
            hash31(((float)id * pos[0] - pos[1]) - pos[2], h1);
            hash31(((float)id * pos[1] + pos[0]) + pos[2], h2);
            const float *lo = b->bmin + 4 * k, *hi = b->bmax + 4 * k;
            const float *R = b->rot ? b->rot + 12 * k : NULL;
            if (!R || R[3] == 0.0f) {
                push_out(pos, lo, hi, radius, h1, h2);
                continue;
            }
            /* oriented: q = R (p - centre), push in [-half, half], p = centre + R^T q */
            float d[3] = {pos[0] - lo[0], pos[1] - lo[1], pos[2] - lo[2]};
            float q[3], nlo[3] = {-hi[0], -hi[1], -hi[2]};
            for (int r = 0; r < 3; ++r) q[r] = (R[4 * r] * d[0] + R[4 * r + 1] * d[1]) + R[4 * r + 2] * d[2];
            if (!push_out(q, nlo, hi, radius, h1, h2)) continue;
            for (int c = 0; c < 3; ++c) pos[c] = lo[c] + ((R[c] * q[0] + R[4 + c] * q[1]) + R[8 + c] * q[2]);
        }
        for (int c = 0; c < 3; ++c) ip[c] = f2i_f(pos[c] * 262144.0f);
    }
}

/* ---- further constraints ---- */
static float fract_p(float x) { return x - floorf(x); }
/* shadertoy 4djSRW hash11 (MIT licence), sphere_collision.comp:24-30 */
static float hash11(float p) {
    p = fract_p(p * 0.1031f);
    p *= p + 33.33f;
    p *= p + p;
    return fract_p(p);
}

/* sphere_collision.comp:42-58 */
void or_sphere_collision(or_fluid *f, const float center[3], float radius, int hollow) {
    for (uint32_t id = 0; id < f->n; ++id) {
        int32_t *ip = f->pos + 4 * (size_t)id;
        float px = (float)ip[0] / 262144.0f, py = (float)ip[1] / 262144.0f, pz = (float)ip[2] / 262144.0f;
        const float r = f->radius[id];
        const float dir = hollow ? -1.0f : 1.0f;
        const float off = dir * (r + hash11((float)id * py + px + pz) * 0.05f);
        const float rx = px - center[0], ry = py - center[1], rz = pz - center[2];
        const float d = sqrtf(rx * rx + ry * ry + rz * rz);
        const float target = radius + off;
        if ((d < target) == (hollow != 0)) continue;
        const float s = target / d;
        ip[0] = f2i_f((center[0] + rx * s) * 262144.0f);
        ip[1] = f2i_f((center[1] + ry * s) * 262144.0f);
        ip[2] = f2i_f((center[2] + rz * s) * 262144.0f);
    }
}

/* inter_particle_collision.comp:33-51 over the ordered pairs of the rows; a Jacobi
 * step: reads the old positions, adds to a copy */
void or_inter_particle_collision(or_fluid *f, const or_neighbors *nb) {
    const uint32_t n = f->n;
    int32_t *old = (int32_t *)malloc(16 * (size_t)(n ? n : 1));
    memcpy(old, f->pos, 16 * (size_t)n);
    for (uint32_t i = 0; i < n; ++i) {
        const int32_t *p = old + 4 * (size_t)i;
        const float r = f->radius[i], im = f->inv_mass[i];
        for (uint32_t e = nb->offsets[i]; e < nb->offsets[i + 1]; ++e) {
            const uint32_t j = nb->idx[e];
            const float rN = f->radius[j];
            if (rN > r || (rN == r && j >= i)) continue;
            const int32_t *q = old + 4 * (size_t)j;
            const float dx = (float)wrap_add(q[0], -p[0]), dy = (float)wrap_add(q[1], -p[1]),
                        dz = (float)wrap_add(q[2], -p[2]);
            const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
            const float ce = dist - (r + rN) * 262144.0f;
            if (ce >= 0.0f) continue;
            const float imN = f->inv_mass[j];
            const float scalar = ce / (im + imN);
            const float a = im * scalar / dist, b = -imN * scalar / dist;
            int32_t *pi = f->pos + 4 * (size_t)i, *pj = f->pos + 4 * (size_t)j;
            pi[0] = wrap_add(pi[0], f2i_f(a * dx));
            pi[1] = wrap_add(pi[1], f2i_f(a * dy));
            pi[2] = wrap_add(pi[2], f2i_f(a * dz));
            pj[0] = wrap_add(pj[0], f2i_f(b * dx));
            pj[1] = wrap_add(pj[1], f2i_f(b * dy));
            pj[2] = wrap_add(pj[2], f2i_f(b * dz));
        }
    }
    free(old);
}

/* generate_glue.comp:30-45, in row order */
uint32_t or_glue_generate(const or_fluid *f, const or_neighbors *nb, uint32_t *g0, uint32_t *g1, uint32_t *gd,
                          uint32_t cap) {
    uint32_t m = 0;
    for (uint32_t i = 0; i < f->n; ++i) {
        const int32_t *p = f->pos + 4 * (size_t)i;
        const float r = f->radius[i];
        for (uint32_t e = nb->offsets[i]; e < nb->offsets[i + 1]; ++e) {
            const uint32_t j = nb->idx[e];
            const float rN = f->radius[j];
            if (rN > r || (rN == r && i >= j)) continue;
            const int32_t *q = f->pos + 4 * (size_t)j;
            const float dx = (float)wrap_add(q[0], -p[0]) / 262144.0f, dy = (float)wrap_add(q[1], -p[1]) / 262144.0f,
                        dz = (float)wrap_add(q[2], -p[2]) / 262144.0f;
            const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
            const float gap = dist - r - rN;
            if (gap > 2.0f * r) continue;
            if (m < cap) {
                g0[m] = i;
                g1[m] = j;
                gd[m] = f2u_f(dist * 262144.0f);
            }
            ++m;
        }
    }
    return m;
}

/* glue.comp:39-54 (integer scatter: order-free) */
void or_glue_apply(or_fluid *f, const uint32_t *g0, const uint32_t *g1, const uint32_t *gd, uint32_t m,
                   float stability) {
    const uint32_t n = f->n;
    int32_t *old = (int32_t *)malloc(16 * (size_t)(n ? n : 1));
    memcpy(old, f->pos, 16 * (size_t)n);  /* every entry reads the positions before any update */
    for (uint32_t k = 0; k < m; ++k) {
        const uint32_t a = g0[k], b = g1[k];
        const int32_t *p0 = old + 4 * (size_t)a, *p1 = old + 4 * (size_t)b;
        const float im0 = f->inv_mass[a], im1 = f->inv_mass[b];
        const float dx = (float)wrap_add(p1[0], -p0[0]), dy = (float)wrap_add(p1[1], -p0[1]),
                    dz = (float)wrap_add(p1[2], -p0[2]);
        const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
        const float ce = dist - (float)gd[k];
        const float scalar = stability * ce / ((im0 + im1) * dist);
        int32_t *q0 = f->pos + 4 * (size_t)a, *q1 = f->pos + 4 * (size_t)b;
        q0[0] = wrap_add(q0[0], f2i_f(im0 * scalar * dx));
        q0[1] = wrap_add(q0[1], f2i_f(im0 * scalar * dy));
        q0[2] = wrap_add(q0[2], f2i_f(im0 * scalar * dz));
        q1[0] = wrap_add(q1[0], f2i_f(-im1 * scalar * dx));
        q1[1] = wrap_add(q1[1], f2i_f(-im1 * scalar * dy));
        q1[2] = wrap_add(q1[2], f2i_f(-im1 * scalar * dz));
    }
    free(old);
}

/* ---- emitter (restates the device's k_emit_plan / k_emit) ---- */
static uint32_t emit_hash(uint32_t seed, uint64_t layer, uint32_t cell, uint32_t axis) {
    uint64_t z = ((uint64_t)seed << 32) ^ (layer * 0x9E3779B97F4A7C15ull) ^ ((uint64_t)cell << 2) ^ axis;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (uint32_t)(z >> 32);
}

static int32_t f2i_trunc(float x) {
    if (!(x == x)) return 0;
    if (x >= 2147483647.0f) return 2147483647;
    if (x <= -2147483648.0f) return (int32_t)(-2147483647 - 1);
    return (int32_t)x;
}

uint32_t or_emit(or_fluid *f, const or_emitter *e, double state[2], float dt, float last_dt, int *overflow) {
    if (overflow) *overflow = 0;
    if (!e->enabled || dt <= 0.0f) return 0;
    const double T = state[0];
    const double layer_dt = (2.0 * (double)e->radius) / (double)e->speed;
    const uint64_t l0 = (uint64_t)ceil(T / layer_dt), l1 = (uint64_t)ceil((T + (double)dt) / layer_dt);
    const uint64_t per_layer = (uint64_t)e->nx * e->nz;
    uint64_t want = (l1 - l0) * per_layer;
    const uint64_t emitted = (uint64_t)state[1];
    if (e->max_particles && emitted + want > e->max_particles) want = e->max_particles > emitted ? e->max_particles - emitted : 0;
    const uint32_t n = f->n;
    const uint64_t room = f->cap > n ? f->cap - n : 0;
    if (want > room) {
        if (overflow) *overflow = 1;
        want = room;
    }
    state[0] = T + (double)dt;
    state[1] = (double)(emitted + want);
    const float jr = e->jitter * e->radius;
    const double d = 2.0 * (double)e->radius;
    const float inv_mass = (float)(1.0 / (d * d * d));
    const int32_t backup_dy = f2i_trunc(e->speed * last_dt * 262144.0f);
    for (uint64_t k = 0; k < want; ++k) {
        const uint64_t layer = l0 + k / per_layer;
        const uint32_t cell = (uint32_t)(k % per_layer), ci = cell / e->nz, cj = cell % e->nz;
        float jit[3];
        for (uint32_t a = 0; a < 3; ++a) {
            const float u = (float)(emit_hash(e->seed, layer, cell, a) >> 8) * 5.9604644775390625e-8f;
            jit[a] = ((2.0f * u) - 1.0f) * jr;
        }
        const double t_l = (double)layer * layer_dt;
        const float dy = (float)((t_l - T) * (double)e->speed);
        const float x = (e->origin[0] + (float)(2u * ci + 1u) * e->radius) + jit[0];
        const float y = (e->origin[1] + dy) + jit[1];
        const float z = (e->origin[2] + (float)(2u * cj + 1u) * e->radius) + jit[2];
        const uint32_t id = n + (uint32_t)k;
        int32_t *p = f->pos + 4 * (size_t)id, *b = f->pos_backup + 4 * (size_t)id;
        p[0] = f2i_trunc(x * 262144.0f);
        p[1] = f2i_trunc(y * 262144.0f);
        p[2] = f2i_trunc(z * 262144.0f);
        p[3] = 0;
        b[0] = p[0];
        b[1] = (int32_t)((uint32_t)p[1] + (uint32_t)backup_dy);
        b[2] = p[2];
        b[3] = 0;
        float *v = f->vel + 4 * (size_t)id;
        v[0] = 0.0f;
        v[1] = -e->speed;
        v[2] = 0.0f;
        v[3] = 0.0f;
        f->inv_mass[id] = inv_mass;
        f->radius[id] = e->radius;
        f->transferring[id] = 0u;
        f->target_radius[id] = e->radius;
        f->kernel_width[id] = e->radius * 4.0f;
        f->boundariness[id] = 1.0f;
        f->boundary_distance[id] = (uint32_t)(e->radius * 262144.0f);
    }
    f->n = n + (uint32_t)want;
    return (uint32_t)want;
}

/* velocity_handling.cpp:15-31; infer_velocity.comp:30-31, apply_acceleration.comp:26-27,
 * apply_velocity.comp:29-30. */
void or_velocity_handling(or_fluid *f, float dt, float last_dt, const float accel[3]) {
    if (dt == 0.0f) {
        memcpy(f->pos_backup, f->pos, 16 * (size_t)f->n);
        return;
    }
    float inv_den = last_dt * 262144.0f;
    float a[3] = {accel[0] * dt, accel[1] * dt, accel[2] * dt};
    float sc = dt * 262144.0f;
    for (uint32_t i = 0; i < f->n; ++i) {
        int32_t *p = f->pos + 4 * (size_t)i;
        int32_t *bk = f->pos_backup + 4 * (size_t)i;
        float *v = f->vel + 4 * (size_t)i;
        for (int c = 0; c < 3; ++c) {
            int32_t d = (int32_t)((uint32_t)p[c] - (uint32_t)bk[c]);
            v[c] = (float)d / inv_den;
        }
        memcpy(bk, p, 16);
        for (int c = 0; c < 3; ++c) {
            v[c] = v[c] + a[c];
            p[c] = wrap_add(p[c], f2i_f(v[c] * sc));
        }
    }
}

/* ------------------------------------------------------------------ */
/* adaptive stages                                                     */
/* ------------------------------------------------------------------ */

/* move_towards of uint_to_float_*.comp (geometric step), FP32. */
static float move_towards_geo(float old_v, float new_v, float step) {
    float dir = (new_v > old_v) ? 1.0f : (new_v < old_v ? -1.0f : 0.0f);
    float result = old_v * (1.0f + step * dir);
    int reached = (old_v < new_v) != (result < new_v);
    return reached ? new_v : result;
}

/* pool.cpp:77-80 -> uint_to_float_with_indexed_lower_bound.comp:31-45, FP32. */
void or_kernel_width_from_boundary_distance(or_fluid *f, const or_settings *s) {
    float factor = s->target_radius_scale_factor / 262144.0f;
    for (uint32_t i = 0; i < f->n; ++i) {
        float value = (float)f->boundary_distance[i] * factor;
        float lb = f->radius[i] * 4.0f;
        value = move_towards_geo(f->kernel_width[i], value, s->kernel_width_adaption_speed);
        f->kernel_width[i] = fmaxf(value, lb);
    }
}

static float len_fixed_f32(const int32_t *p, const int32_t *q) {
    float d[3];
    for (int c = 0; c < 3; ++c) d[c] = (float)(int32_t)((uint32_t)q[c] - (uint32_t)p[c]) / 262144.0f;
    return sqrtf((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
}

/* spread_kernel_width.cpp:12-26 -> kernel_width_init.comp, kernel_width.comp,
 * uint_to_float_but_gradual.comp; FP32.  Prunes nb rows in place (order kept). */
void or_spread_kernel_width(or_fluid *f, or_neighbors *nb, const or_settings *s) {
    uint32_t n = f->n;
    uint32_t *ukw = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    for (uint32_t i = 0; i < n; ++i) {
        float tr = s->base_kernel_width_on_target_radius ? f->target_radius[i] : 0.0f;
        float ok = fmaxf(f->radius[i], tr) * 4.0f;
        ukw[i] = f2u_f(ok * 262144.0f);
    }
    uint32_t w = 0;
    uint32_t row_start = 0;
    for (uint32_t i = 0; i < n; ++i) {
        float tr = s->base_kernel_width_on_target_radius ? f->target_radius[i] : 0.0f;
        float ok = fmaxf(f->radius[i], tr) * 4.0f;
        float cut = ok > f->kernel_width[i] ? ok : f->kernel_width[i];
        uint32_t b = row_start, e = nb->offsets[i + 1];
        row_start = e;
        nb->offsets[i] = w;
        for (uint32_t k = b; k < e; ++k) {
            uint32_t j = nb->idx[k];
            float dist = len_fixed_f32(f->pos + 4 * (size_t)i, f->pos + 4 * (size_t)j);
            float dfk = dist - ok;
            float t = dfk / (ok * 0.5f);
            float infl = fmaxf(0.0f, 1.0f - fmaxf(0.0f, t));
            uint32_t v = f2u_f((ok * infl) * 262144.0f);
            if (v > ukw[j]) ukw[j] = v;
            if (dist <= cut) nb->idx[w++] = j;
        }
    }
    nb->offsets[n] = w;
    for (uint32_t i = 0; i < n; ++i) {
        float value = (float)ukw[i] * (1.0f / 262144.0f);
        value = move_towards_geo(f->kernel_width[i], value, s->kernel_width_adaption_speed);
        f->kernel_width[i] = fmaxf(value, -INFINITY);
    }
    free(ukw);
}

static uint32_t isqrt_u64(uint64_t x) {  /* floor(sqrt(x)) */
    uint64_t r = (uint64_t)sqrt((double)x);
    while (r * r > x) --r;
    while ((r + 1) * (r + 1) <= x) ++r;
    return (uint32_t)r;
}
static uint32_t fixed_dist(const int32_t *p, const int32_t *q) {  /* C5 */
    uint64_t s = 0;
    for (int c = 0; c < 3; ++c) {
        int64_t d = (int64_t)q[c] - (int64_t)p[c];
        s += (uint64_t)(d * d);
    }
    return isqrt_u64(s);
}

/* Constant of the split test, pow(2.0, 1.0 / DIMENSIONS) * 0.99 (find_split_and_merge_3.comp:90). */
static float split_constant(void) { return (float)(cbrt(2.0) * 0.99); }

/* update_transfers::apply (update_transfers.cpp:14-71). */
void or_update_transfers(or_fluid *f, const or_neighbors *nb, or_transfers *t, const or_settings *s,
                         uint32_t max_transfers) {
    uint32_t n = f->n;
    uint32_t *old_bd = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    uint32_t *min_nd = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    uint32_t *nearest = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    uint32_t *splits = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    memcpy(old_bd, f->boundary_distance, n * sizeof(uint32_t));
    /* find_split_and_merge_1.comp:17-35 */
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t bd = UINT32_MAX, md = UINT32_MAX;
        for (uint32_t e = nb->offsets[i]; e < nb->offsets[i + 1]; ++e) {
            uint32_t j = nb->idx[e];
            uint32_t d = fixed_dist(f->pos + 4 * (size_t)i, f->pos + 4 * (size_t)j);
            uint32_t c = old_bd[j] + d;
            if (c < bd) bd = c;
            if (d < md) md = d;
        }
        f->boundary_distance[i] = bd;
        min_nd[i] = md;
    }
    /* find_split_and_merge_2.comp:19-38 (C6) */
    for (uint32_t i = 0; i < n; ++i) {
        nearest[i] = UINT32_MAX;
        for (uint32_t e = nb->offsets[i]; e < nb->offsets[i + 1]; ++e) {
            uint32_t j = nb->idx[e];
            if (fixed_dist(f->pos + 4 * (size_t)i, f->pos + 4 * (size_t)j) == min_nd[i] && j < nearest[i]) nearest[i] = j;
        }
    }
    /* find_split_and_merge_3.comp:46-122, FP32, claims in index order (C7) */
    const float C = split_constant();
    const float sf = s->target_radius_scale_factor;
    uint32_t n_splits = 0, n_merges = 0;
    uint32_t *msrc = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    uint32_t *mtgt = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    for (uint32_t id = 0; id < n; ++id) {
        const int32_t *p = f->pos + 4 * (size_t)id;
        float radius = f->radius[id];
        float bdist = (float)f->boundary_distance[id] / 262144.0f;
        float bness = f->boundariness[id];
        uint32_t nn = nearest[id];
        int has_nn = nn != UINT32_MAX;
        float nnd = 0.0f, nnr = 0.0f;
        int nn_larger = 0;
        if (has_nn) {
            float d[3];
            for (int c = 0; c < 3; ++c) d[c] = (float)(int32_t)((uint32_t)f->pos[4 * (size_t)nn + c] - (uint32_t)p[c]);
            nnd = sqrtf((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]) / 262144.0f;
            nnr = f->radius[nn];
            nn_larger = nnr > radius || (nnr == radius && nn > id);
        }
        float target;
        if (s->update_target_radius) {
            if (s->base_kernel_width_on_boundary_distance) {
                target = (sf / (4.0f + 4.0f * sf)) * bdist;
                target = fmaxf(target, s->smallest_target_radius);
            } else {
                target = s->smallest_target_radius + fmaxf(0.0f, (bdist - s->target_radius_offset) * sf);
            }
            f->target_radius[id] = target;
        } else {
            target = f->target_radius[id];
        }
        bness = bness >= 1.0f ? 1.0f : 0.0f;
        f->boundary_distance[id] = f2u_f((bdist * (1.0f - bness) + radius * bness) * 262144.0f);
        f->boundariness[id] = bness;

        int split = s->split && (target * C <= radius);
        int merge = s->merge && has_nn && nnd < radius &&
                    (radius * radius * radius + nnr * nnr * nnr <= target * target * target);
        if (!merge && !split) continue;
        uint32_t src = (merge && nn_larger) ? nn : id;
        uint32_t tgt = (merge && nn_larger) ? id : nn;
        if (f->transferring[src] == 1u) continue;
        f->transferring[src] = 1u;
        if (merge) {
            if (f->transferring[tgt] == 1u) {
                f->transferring[src] = 0u;
                continue;
            }
            f->transferring[tgt] = 1u;
            msrc[n_merges] = src;
            mtgt[n_merges] = tgt;
            n_merges++;
        } else {
            splits[n_splits++] = id;
        }
    }
    /* C7 capacity: keep the first accepted merges in index order, release the rest. */
    {
        uint32_t room = max_transfers > t->n ? max_transfers - t->n : 0u;
        if (room > t->cap - t->n) room = t->cap - t->n;
        for (uint32_t k = 0; k < n_merges; ++k) {
            if (k < room) {
                t->source[t->n] = msrc[k];
                t->target[t->n] = mtgt[k];
                t->time_left[t->n] = fmaxf(0.0001f, s->merge_duration);
                t->n++;
            } else {
                f->transferring[msrc[k]] = 0u;
                f->transferring[mtgt[k]] = 0u;
            }
        }
    }
    free(msrc); free(mtgt);
    /* remove_impossible_splits.comp:29-45 */
    if (s->split) {
        uint32_t keep = n_splits;
        uint32_t free_t = max_transfers > t->n ? max_transfers - t->n : 0u;
        uint32_t free_p = f->cap > n ? f->cap - n : 0u;
        if (keep > free_t) keep = free_t;
        if (keep > free_p) keep = free_p;
        for (uint32_t k = keep; k < n_splits; ++k) f->transferring[splits[k]] = 0u;
        /* indexed_list::duplicate_these (indexed_list.h:140-152) + initialize_split_particles.comp */
        uint32_t *edit = (uint32_t *)malloc((size_t)(n + keep ? n + keep : 1) * sizeof(uint32_t));
        for (uint32_t i = 0; i < n; ++i) edit[i] = i;
        for (uint32_t k = 0; k < keep; ++k) edit[n + k] = splits[k];
        fluid_apply_edit(f, edit, n + keep);
        for (uint32_t k = 0; k < keep; ++k) {
            uint32_t d = n + k;
            float r = f->radius[d];
            f->pos[4 * (size_t)d] = wrap_add(f->pos[4 * (size_t)d], f2i_f((r * 262144.0f) * 0.1f));
            f->radius[d] = 0.0f;
            f->inv_mass[d] = INFINITY;
            t->source[t->n] = splits[k];
            t->target[t->n] = d;
            t->time_left[t->n] = -s->split_duration;
            t->n++;
        }
        free(edit);
    } else {
        for (uint32_t k = 0; k < n_splits; ++k) f->transferring[splits[k]] = 0u;
    }
    free(old_bd); free(min_nd); free(nearest); free(splits);
}

/* particle_transfer::apply (particle_transfer.cpp:10-28) + particle_transfer.comp:31-85.
 * Volumes and masses in FP64; the time-left countdown in FP32 so that the step at
 * which a transfer finishes matches the FP32 device path exactly. */
void or_particle_transfer(or_fluid *f, or_transfers *t, float dt) {
    uint32_t n = f->n;
    uint32_t *del_p = (uint32_t *)malloc((t->n ? t->n : 1) * sizeof(uint32_t));
    uint8_t *del_t = (uint8_t *)calloc(t->n ? t->n : 1, 1);
    uint32_t nd = 0;
    for (uint32_t k = 0; k < t->n; ++k) {
        float tt = t->time_left[k];
        float att = fabsf(tt);
        float ttl = dt > att ? dt : att;
        int merge = tt > 0.0f;
        uint32_t S = t->source[k], T = t->target[k];
        double rS = f->radius[S], rT = f->radius[T];
        double imS = f->inv_mass[S], imT = f->inv_mass[T];
        double volS = rS * rS * rS, volT = rT * rT * rT;
        double factor = merge ? fmin(1.0, (double)dt / (double)ttl)
                              : (double)dt * (volS - volT) / (2.0 * (double)ttl * volS);
        double tv = factor * volS;
        f->inv_mass[S] = (float)(imS / (1.0 - factor));
        if (isinf(imT)) f->inv_mass[T] = (float)(imS / factor); /* C9 */
        else f->inv_mass[T] = (float)(imS * imT / (imS + factor * imT));
        f->radius[S] = (float)cbrt(volS - tv);
        f->radius[T] = (float)cbrt(volT + tv);
        t->time_left[k] = (ttl - dt) * (merge ? 1.0f : -1.0f);
        if (ttl == dt) {
            if (merge) del_p[nd++] = S;
            else del_t[k] = 1;
            f->transferring[S] = 0u;
            f->transferring[T] = 0u;
        }
    }
    /* deleteTransferList.delete_these() */
    uint32_t m = 0;
    for (uint32_t k = 0; k < t->n; ++k) {
        if (del_t[k]) continue;
        t->source[m] = t->source[k];
        t->target[m] = t->target[k];
        t->time_left[m] = t->time_left[k];
        ++m;
    }
    t->n = m;
    /* deleteParticleList.delete_these() */
    if (nd) {
        uint32_t *edit = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
        uint32_t nn = or_delete_edit_list(n, del_p, nd, edit);
        fluid_apply_edit(f, edit, nn);
        transfers_remap(t, edit, nn, n);
        free(edit);
    }
    free(del_p); free(del_t);
}

/* Global reductions, FP64: mass, volume, mean compression error (no reference counterpart). */
void or_reduce(const or_fluid *f, double out[3]) {
    double m = 0.0, v = 0.0;
    for (uint32_t i = 0; i < f->n; ++i) {
        m += 1.0 / (double)f->inv_mass[i];
        double r = f->radius[i];
        v += r * r * r;
    }
    out[0] = m;
    out[1] = v;
    out[2] = 0.0;
}

/* Mean density error on the substep's neighbour list at the current positions:
 * out[0] = mean max(0, rho_i / rho0_i - 1), out[1] = mean |rho_i / rho0_i - 1|
 * (densities as incompressibility_0/1 compute them; rho0_i^-1 as
 * incompressibility_2.comp:81).  No reference counterpart. */
void or_density_error(const or_fluid *f, const or_neighbors *nb, const or_settings *s, double out[2]) {
    const double R = OR_POS_RESOLUTION;
    double e1 = 0.0, e2 = 0.0;
    for (uint32_t i = 0; i < f->n; ++i) {
        const int32_t *p = f->pos + 4 * (size_t)i;
        double kw = f->kernel_width[i];
        double zero[3] = {0, 0, 0};
        uint32_t dens = f2u(or_kernel_height(s->height_kernel_id, zero, kw) / f->inv_mass[i] * R);
        for (uint32_t e = nb->offsets[i]; e < nb->offsets[i + 1]; ++e) {
            const int32_t *q = f->pos + 4 * (size_t)nb->idx[e];
            double d[3];
            for (int c = 0; c < 3; ++c) d[c] = (double)(int32_t)((uint32_t)q[c] - (uint32_t)p[c]) / R;
            dens += f2u(or_kernel_height(s->height_kernel_id, d, kw) / f->inv_mass[nb->idx[e]] * R);
        }
        double ird = pow(2.0 * (double)f->radius[i], 3.0) * (double)f->inv_mass[i];
        double ratio = (double)dens / R * ird - 1.0;
        e1 += ratio > 0.0 ? ratio : 0.0;
        e2 += fabs(ratio);
    }
    out[0] = f->n ? e1 / f->n : 0.0;
    out[1] = f->n ? e2 / f->n : 0.0;
}

/* pool::update (pool.cpp:67-106). */
uint64_t or_substep(or_fluid *f, or_transfers *t, or_neighbors *nb, const or_boxes *b, or_scene *sc, float dt) {
    const or_settings *s = &sc->settings;
    or_velocity_handling(f, dt, sc->last_dt, sc->accel);
    if (dt != 0.0f) sc->last_dt = dt;
    if (!s->basic_pbf && (s->merge || s->split)) or_particle_transfer(f, t, dt);
    if (!s->basic_pbf && s->base_kernel_width_on_boundary_distance) or_kernel_width_from_boundary_distance(f, s);
    float scale = (s->basic_pbf || s->base_kernel_width_on_boundary_distance) ? 1.0f : 1.5f;
    uint64_t pairs = sc->search_method == 3 ? or_neighborhood_binary_search(f, t, scale, nb, NULL, NULL)
                                            : or_neighborhood_green(f, t, scale, sc->minp, sc->maxp, sc->log2res, nb,
                                                                    NULL, NULL);
    if (pairs > nb->cap) return pairs;
    if (!s->basic_pbf && !s->base_kernel_width_on_boundary_distance) or_spread_kernel_width(f, nb, s);
    for (int it = 0; it < s->solver_iterations; ++it) {
        or_box_collision(f, b);
        if (s->density_error_target > 0.0f) {
            /* the device measures the error in each density pass and stops before
             * correcting once it is at most the target */
            double e[2];
            or_density_error(f, nb, s, e);
            if (e[0] <= (double)s->density_error_target) break;
        }
        or_incompressibility_apply(f, nb, s, NULL);
    }
    if (!s->basic_pbf) or_update_transfers(f, nb, t, s, sc->max_transfers);
    return pairs;
}
