/*
 * apbf_oracle.h -- CPU restatement of the adaptive PBF substep of cg-tuwien/APBF.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the correctness oracle for the CUDA
 * implementation in apbf_gb300/.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load it, and only as the parity reference or
 * as the timed CPU baseline; the product path never calls it.
 *
 * The reference runs its physics only as GLSL compute shaders through Vulkan; it
 * has no CPU implementation and cannot be built here (MSVC project, un-vendored
 * Gears-Vk submodule, no graphics API).  This file restates the shader math in
 * plain C, single-threaded:
 *   - FP64 for the smoothing kernels, the density / lambda solve, kernel widths,
 *     split/merge decisions and particle transfer (the "FP64 oracle");
 *   - exact FP32 emulation (no FMA contraction, build with -ffp-contract=off) for
 *     the stages whose reference arithmetic is only meaningful at FP32: the box
 *     collision hash jitter (box_collision.comp:20-25, a fract()-based hash) and
 *     velocity integration (infer_velocity.comp, apply_acceleration.comp,
 *     apply_velocity.comp);
 *   - exact integer arithmetic for Morton codes, sort permutations, cell ranges,
 *     neighbour predicates, prefix sums, list edits and split/merge claims.
 *
 * Canonical rules where the reference is racy or undefined are listed in
 * apbf_oracle.c next to the code that implements them.
 *
 * Pinning: the primitives and list edits are checked against every known-answer
 * vector of the reference's source/test.cpp (tests/golden).  The reference has no
 * test of its physics and cannot be run here, so for the neighbour search,
 * kernels, incompressibility, kernel width, split/merge and transfer the oracle's
 * parity with the reference is unpinned: it is a line-by-line restatement of the
 * cited shaders, self-checked only.
 *
 * Every fluid array is indexed by the same particle id (hidden-list order equals
 * fluid order, as it does in every reference scene after the neighbour sort).
 */
#ifndef APBF_ORACLE_H
#define APBF_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OR_POS_RESOLUTION 262144.0      /* cpu_gpu_shared_config.h:7  */
#define OR_KERNEL_SCALE 4.0             /* cpu_gpu_shared_config.h:14 */
#define OR_KW_PROPAGATION 0.5           /* cpu_gpu_shared_config.h:15 */

/* Mirrors apbf_settings (cpu_gpu_shared_config.h:74-94) plus the host-side
 * pbd::settings that steer the substep (settings.cpp:5-31). */
typedef struct or_settings {
    int32_t height_kernel_id;
    int32_t gradient_kernel_id;
    int32_t merge;
    int32_t split;
    int32_t base_kernel_width_on_target_radius;
    int32_t base_kernel_width_on_boundary_distance;
    int32_t update_target_radius;
    int32_t update_boundariness;
    int32_t boundariness_calculation_method;
    int32_t basic_pbf;
    int32_t solver_iterations;
    int32_t pad0;
    float boundariness_adaption_speed;
    float kernel_width_adaption_speed;
    float boundariness_self_grad_length_factor;
    float boundariness_underpressure_factor;
    float merge_duration;
    float split_duration;
    float smallest_target_radius;
    float target_radius_offset;
    float target_radius_scale_factor;
    float density_error_target; /* > 0: stop the iterations once the error is at most this */
    float pad1[2];
} or_settings;

/* Particle + fluid state, structure of arrays.  pos / pos_backup are ivec4
 * (x, y, z, pad) in 2^18 fixed point, vel is vec4. */
typedef struct or_fluid {
    uint32_t n;
    uint32_t cap;
    int32_t *pos;
    float *vel;
    float *inv_mass;
    float *radius;
    int32_t *pos_backup;
    uint32_t *transferring;
    float *target_radius;
    float *kernel_width;
    float *boundariness;
    uint32_t *boundary_distance;
} or_fluid;

/* Transfer list (hidden_transfers, list_definitions.h:16-18): particle ids. */
typedef struct or_transfers {
    uint32_t n;
    uint32_t cap;
    uint32_t *source;
    uint32_t *target;
    float *time_left;
} or_transfers;

/* Neighbour list in CSR form: row i holds every j with |x_j - x_i| <= R_i,
 * sorted ascending.  The reference's unordered uvec2 pair list
 * (list_definitions.h:20) is this list flattened. */
typedef struct or_neighbors {
    uint32_t n;
    uint32_t cap;        /* capacity of idx */
    uint32_t *offsets;   /* n + 1 */
    uint32_t *idx;
} or_neighbors;

/* Axis-aligned boxes (user_controlled_boxes), vec4 min / vec4 max. */
typedef struct or_boxes {
    uint32_t n;
    const float *bmin;
    const float *bmax;
    /* NULL, or 12 floats per box: the rows of its rotation (its local axes); row 0
     * element 3 != 0 marks an oriented box, whose bmin is its centre and bmax its
     * half extents (no reference counterpart: the reference's boxes are axis-aligned). */
    const float *rot;
} or_boxes;

/* ---- primitives (algorithms.cpp) ---- */
void or_prefix_sum_inclusive(const uint32_t *in, uint32_t *out, size_t n);
void or_sort_pairs_stable(const uint32_t *keys, const uint32_t *vals, size_t n,
                          uint32_t *out_keys, uint32_t *out_vals);

/* ---- list edits (gpu_list.h, indexed_list.h) ---- */
void or_apply_edit_u32(const uint32_t *src, const uint32_t *edit, size_t n_edit, uint32_t stride_words,
                       uint32_t *dst);
uint32_t or_delete_edit_list(uint32_t n_hidden, const uint32_t *deleted, uint32_t n_deleted, uint32_t *edit);
uint32_t or_remap_index_list(const uint32_t *list, uint32_t n_list, const uint32_t *edit, uint32_t n_edit,
                             uint32_t n_hidden_old, uint32_t *out, uint32_t *new_edit, uint32_t max_out);

/* ---- neighbour search (neighborhood_green) ---- */
void or_fixed_bounds(const float minp[3], const float maxp[3], int64_t out_min[3], int64_t out_max[3]);
uint32_t or_cell_coord(int64_t x, int64_t xmin, int64_t xmax, uint32_t log2res);
uint32_t or_morton(const uint32_t c[3], uint32_t log2res);
void or_position_keys(const int32_t *pos4, size_t n, const float minp[3], const float maxp[3],
                      uint32_t log2res, uint32_t *keys);
void or_cell_ranges(const uint32_t *sorted_keys, size_t n, uint32_t ncells, uint32_t *start, uint32_t *end);
int64_t or_range_fixed(float kernel_width, float range_scale);
/* Returns the total number of pairs; if it exceeds nb->cap the rows are not written. */
uint64_t or_neighbors_build(const int32_t *pos4, const float *range, float range_scale, size_t n,
                            const float minp[3], const float maxp[3], uint32_t log2res,
                            const uint32_t *cell_start, const uint32_t *cell_end, or_neighbors *nb);
uint64_t or_neighbors_brute(const int32_t *pos4, const float *range, float range_scale, size_t n,
                            or_neighbors *nb);
/* Full neighborhood_green::apply: keys, stable sort, reorder of every attribute,
 * cell ranges, neighbour rows.  perm_out (may be NULL) receives the sort
 * permutation (new id -> old id).  Transfers are remapped. Returns pair count. */
uint64_t or_neighborhood_green(or_fluid *f, or_transfers *t, float range_scale, const float minp[3],
                               const float maxp[3], uint32_t log2res, or_neighbors *nb,
                               uint32_t *perm_out, uint32_t *keys_out);
/* neighborhood_binary_search (calculate_position_code.comp, neighborhood_binary_search.comp):
 * the 96-bit position code, the rows over a sorted code list, and the whole apply. */
void or_position_code96(const int32_t *p, uint32_t out[3]);
uint64_t or_neighbors_binary_search(const int32_t *pos4, const uint32_t *codes3, const float *range,
                                    float range_scale, size_t n, or_neighbors *nb);
uint64_t or_neighborhood_binary_search(or_fluid *f, or_transfers *t, float range_scale, or_neighbors *nb,
                                       uint32_t *perm_out, uint32_t *codes_out);

/* ---- smoothing kernels (kernels.glsl) ---- */
double or_kernel_height(int id, const double r[3], double kw);
void or_kernel_gradient(int id, const double r[3], double kw, double out[3]);

/* ---- incompressibility (incompressibility_0..3.comp) ---- */
typedef struct or_incomp_out {
    uint32_t *density;      /* n, fixed point 2^18 */
    int32_t *grad_sum;      /* 3n */
    uint32_t *sq_grad_sum;  /* n */
    float *lambda;          /* n */
    /* Learned warm start (no reference counterpart): per-particle velocity
     * divergence x density, sum_j m_j (v_j - v_i) . gradW_ij, of this pass (out);
     * and, when non-NULL, the lambda that replaces the computed one in this
     * pass's position update (in). */
    float *divergence;      /* n */
    const float *lambda_in; /* n */
    /* Projected pass of a warm-started substep (no reference counterpart): when
     * non-NULL, the sum of the lambdas applied to each particle earlier in the
     * substep (<= 0); a positive lambda is then applied up to minus that sum
     * (pull-back).  `applied` (out) receives the lambda each particle applied. */
    const float *projected_acc; /* n */
    float *applied;             /* n */
} or_incomp_out;
void or_incompressibility_apply(or_fluid *f, const or_neighbors *nb, const or_settings *s,
                                or_incomp_out *out);

/* ---- substep glue ---- */
void or_box_collision(or_fluid *f, const or_boxes *b);

/* Further constraint operators (sphere_collision.comp, inter_particle_collision.comp,
 * generate_glue.comp + glue.comp), plain FP32 arithmetic in the shaders' order. */
void or_sphere_collision(or_fluid *f, const float center[3], float radius, int hollow);
void or_inter_particle_collision(or_fluid *f, const or_neighbors *nb);
/* glue pairs of the rows in row order; returns the count (at most cap written) */
uint32_t or_glue_generate(const or_fluid *f, const or_neighbors *nb, uint32_t *g0, uint32_t *g1, uint32_t *gd,
                          uint32_t cap);
void or_glue_apply(or_fluid *f, const uint32_t *g0, const uint32_t *g1, const uint32_t *gd, uint32_t m,
                   float stability);

/* Emitter (no reference counterpart; the device's apbf_set_emitter / the first
 * stage of apbf_substep): appends the lattice layers that cross the emission plane
 * during dt.  state: [0] stream time, [1] particles emitted so far. */
typedef struct or_emitter {
    float origin[3];
    float radius;
    uint32_t nx, nz;
    float speed;
    float jitter;
    uint32_t seed;
    uint32_t max_particles;
    uint32_t enabled;
    uint32_t pad;
} or_emitter;
/* returns the number appended; sets *overflow when the capacity cut the emission */
uint32_t or_emit(or_fluid *f, const or_emitter *e, double state[2], float dt, float last_dt, int *overflow);
void or_velocity_handling(or_fluid *f, float dt, float last_dt, const float accel[3]);

/* ---- adaptive stages ---- */
void or_kernel_width_from_boundary_distance(or_fluid *f, const or_settings *s);
void or_spread_kernel_width(or_fluid *f, or_neighbors *nb, const or_settings *s);
void or_update_transfers(or_fluid *f, const or_neighbors *nb, or_transfers *t, const or_settings *s,
                         uint32_t max_transfers);
void or_particle_transfer(or_fluid *f, or_transfers *t, float dt);

/* ---- reductions ---- */
void or_reduce(const or_fluid *f, double out[3]);
void or_density_error(const or_fluid *f, const or_neighbors *nb, const or_settings *s, double out[2]);

/* ---- whole substep (pool.cpp:67-106) ---- */
typedef struct or_scene {
    or_settings settings;
    float minp[3];
    float maxp[3];
    uint32_t log2res;
    float accel[3];
    float last_dt;
    uint32_t max_transfers;
    uint32_t search_method; /* NEIGHBORHOOD_TYPE numbering: 3 binary search, else Green */
} or_scene;
uint64_t or_substep(or_fluid *f, or_transfers *t, or_neighbors *nb, const or_boxes *b, or_scene *sc, float dt);

#ifdef __cplusplus
}
#endif
#endif
