/*
 * apbf_gb300.h -- C ABI of the GB300-native adaptive PBF substep.
 *
 * This is the drop-in boundary for the hot path of cg-tuwien/APBF: the stage
 * objects that scene code calls once per frame (pool::update, source/pool.cpp:67-106)
 * -- neighbourhood search, incompressibility solve, kernel-width adaptation,
 * split/merge and particle transfer -- plus the parallel primitives they use.
 *
 * Conventions, kept from the reference's device list model (source/gpu_list.h,
 * source/gpu_list_data.h:8-14):
 *  - Particle data is structure-of-arrays in device memory.  Positions are ivec4
 *    (x, y, z, pad) in 2^18 fixed point (cpu_gpu_shared_config.h:7); velocities
 *    are vec4.
 *  - Every list length lives in device memory (a uint32_t), so a whole substep
 *    runs without a host round trip and can be captured in a CUDA graph.
 *    Capacities are fixed at apbf_create time (the reference's "requested length").
 *  - The context owns all list buffers, like gpu_list owns pooled buffers.  Device
 *    pointers returned by the *_view functions stay valid until the next call that
 *    edits the lists (a neighbourhood search reorders particles into the alternate
 *    buffer set; particle transfer and split/merge change lengths), exactly as
 *    gpu_list::buffer() is "valid until another function of this object is called"
 *    (source/indexed_list.h:40).
 *  - Every stage call is asynchronous on the given stream and never synchronises.
 *    Overflows and device-side failures are recorded in a device status word;
 *    apbf_get_status() reads it (and synchronises the stream).
 *  - Units are the reference's: lengths in particle radii of the smallest particle
 *    (scenes use radius 1, source/main.cpp:63-68), kernel width 4 radii.
 *
 * All functions return an apbf_status.  No function throws or aborts.
 */
#ifndef APBF_GB300_H
#define APBF_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define APBF_ABI_VERSION 1u
#define APBF_POS_RESOLUTION 262144.0f /* cpu_gpu_shared_config.h:7 */
#define APBF_KERNEL_SCALE 4.0f        /* cpu_gpu_shared_config.h:14 */
#define APBF_MAX_TRANSFERS 10000u     /* cpu_gpu_shared_config.h:17 */
#define APBF_MAX_BOXES 64u

typedef enum apbf_status {
    APBF_OK = 0,
    APBF_ERR_INVALID_ARG = 1,
    APBF_ERR_CAPACITY = 2,   /* a list overflowed; apbf_status_info.required_* says how much was needed */
    APBF_ERR_NONFINITE = 3,  /* NaN / inf found in a position or lambda */
    APBF_ERR_SPIN_LIMIT = 4, /* a device-side wait gave up (bounded spin) */
    APBF_ERR_CUDA = 5,       /* a CUDA runtime call failed; apbf_last_error() has the text */
    APBF_ERR_NOT_BUILT = 6
} apbf_status;

/* Device status flags (bit set in apbf_status_info.flags). */
#define APBF_FLAG_NEIGHBOR_OVERFLOW 0x1u
#define APBF_FLAG_TRANSFER_OVERFLOW 0x2u
#define APBF_FLAG_PARTICLE_OVERFLOW 0x4u
#define APBF_FLAG_SPIN_LIMIT 0x8u
#define APBF_FLAG_NONFINITE 0x10u
#define APBF_FLAG_GRID_OVERFLOW 0x20u

/* Run-time switches: apbf_settings UBO (cpu_gpu_shared_config.h:74-94) plus the
 * host-side pbd::settings that steer the substep (source/settings.cpp:5-31).
 * apbf_default_settings() returns the reference defaults. */
typedef struct apbf_settings {
    int32_t height_kernel_id;   /* 0 cubic, 1 Gauss (default), 2 poly6, 3 cone, 4 quadratic spike */
    int32_t gradient_kernel_id; /* 0 cubic, 1 Gauss (default), 2 spiky, 3 cone, 4 quadratic spike */
    int32_t merge;
    int32_t split;
    int32_t base_kernel_width_on_target_radius;
    int32_t base_kernel_width_on_boundary_distance;
    int32_t update_target_radius;
    int32_t update_boundariness;
    int32_t boundariness_calculation_method; /* 0 gradient, 1 centre of mass, 2 gradient + filter */
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
    /* Not in the reference: when > 0, the Jacobi iterations of apbf_substep stop as
     * soon as the mean compression error max(0, rho/rho0 - 1) measured by a density
     * pass is at most this value; solver_iterations is then the maximum. */
    float density_error_target;
    float pad1[2];
} apbf_settings;

/* Capacities (the reference's requested lengths, source/pool.cpp:7-15). */
typedef struct apbf_config {
    uint32_t particle_capacity;
    uint32_t max_neighbors;     /* neighbour row capacity per particle */
    uint32_t transfer_capacity; /* APBF_MAX_TRANSFERS in the reference */
    uint32_t max_log2res;       /* largest grid resolution (bits per axis) the context may be asked for */
    int32_t device;
    uint32_t reserved[3];
} apbf_config;

/* Scene parameters used by apbf_substep (pool::update, source/pool.cpp:67-106) and
 * by neighborhood_green::set_position_range (source/neighborhood_green.h:13). */
typedef struct apbf_scene {
    float min_pos[3];
    float max_pos[3];
    uint32_t log2res;
    float acceleration[3];
} apbf_scene;

/* Particle and fluid lists: hidden_particles + fluid (source/list_definitions.h:9-14),
 * one entry per particle (the fluid index list is the identity after every sort). */
typedef struct apbf_fluid_view {
    uint32_t capacity;
    uint32_t *d_length;
    int32_t *position;     /* int4; w is reserved: the neighbourhood search stores the particle's
                              mass there for the incompressibility passes */
    float *velocity;       /* float4 */
    float *inverse_mass;
    float *radius;
    int32_t *pos_backup;   /* int4 */
    uint32_t *transferring;
    float *target_radius;
    float *kernel_width;
    float *boundariness;
    uint32_t *boundary_distance;
} apbf_fluid_view;

/* The particle lists in host memory (structure of arrays, one entry per particle);
 * a null field is not copied.  lambda_prev is the warm start's per-particle history
 * (no reference counterpart). */
typedef struct apbf_host_fluid {
    int32_t *position;     /* int4 (w: library scratch, see apbf_fluid_view) */
    float *velocity;       /* float4 */
    float *inverse_mass;
    float *radius;
    int32_t *pos_backup;   /* int4 */
    uint32_t *transferring;
    float *target_radius;
    float *kernel_width;
    float *boundariness;
    uint32_t *boundary_distance;
    float *lambda_prev;
} apbf_host_fluid;

/* transfers = indexed_list<hidden_transfers> (source/list_definitions.h:16-18). */
typedef struct apbf_transfers_view {
    uint32_t capacity;
    uint32_t *d_length;
    uint32_t *source;
    uint32_t *target;
    float *time_left; /* > 0 merge, <= 0 split (particle_transfer.comp:37-39) */
} apbf_transfers_view;

/* Neighbour rows, column-major ("transposed ELL"): the k-th neighbour of particle i
 * is index[k * row_stride + i], for k < count[i].  This replaces the reference's
 * unordered uvec2 pair list (source/list_definitions.h:20); apbf_export_pairs()
 * produces that list. */
typedef struct apbf_neighbors_view {
    uint32_t row_stride;
    uint32_t max_per_row;
    uint32_t *count;
    uint32_t *index;
    unsigned long long *d_total; /* total pairs of the last search */
} apbf_neighbors_view;

typedef struct apbf_status_info {
    uint32_t flags;
    uint32_t required_neighbors; /* largest row seen when APBF_FLAG_NEIGHBOR_OVERFLOW is set */
    uint32_t required_transfers;
    uint32_t required_particles;
    unsigned long long pairs;    /* pairs of the last neighbourhood search */
    uint32_t density_passes;     /* density passes executed since the status was last cleared */
    uint32_t converged_substeps; /* substeps whose density error met density_error_target, same period */
    uint32_t spin_where;         /* with APBF_ERR_SPIN_LIMIT: the wait that gave up: 1 sort look-back, 2 scan
                                    look-back, 3 persistent-solve grid barrier, 4 batched-solve grid barrier */
    uint32_t reserved;
} apbf_status_info;

/* Launch shapes of the context's kernels (no reference counterpart: the
 * reference's workgroup sizes are fixed in its shaders).  Results do not depend
 * on them. */
typedef struct apbf_tuning {
    uint32_t gather_lanes;        /* threads per particle in the density and position passes: 1, 2, 4 or 8 */
    uint32_t pass_block;          /* threads per block of those passes: 128 or 256 */
    uint32_t pass_blocks_per_sm;  /* their grid: up to this many blocks per SM (1..8) */
    uint32_t reserved0;           /* must be 0 */
    uint32_t filter_in_density;   /* 1: the boundariness filter always runs in the density pass (else, with
                                     symmetric rows and the Gauss kernel, in the position pass) */
    uint32_t sort_digit_bits;     /* radix sort digit width: 6, 7 or 8 bits per pass (0: 8); same order */
    uint32_t search_log2res;      /* apbf_substep's search grid: 2^L cells per axis over the scene's box
                                     (0: the scene's log2res); the same neighbour sets, particle order
                                     and row order follow the grid */
    uint32_t reserved;
} apbf_tuning;

typedef struct apbf_ctx apbf_ctx;

/* ---- lifetime and configuration ---- */
uint32_t apbf_abi_version(void);
const char *apbf_last_error(void);
void apbf_default_settings(apbf_settings *out);                         /* source/settings.cpp:5-31 */
apbf_status apbf_create(const apbf_config *cfg, apbf_ctx **out);
apbf_status apbf_destroy(apbf_ctx *ctx);
apbf_status apbf_set_settings(apbf_ctx *ctx, const apbf_settings *s);   /* settings.cpp:66-90 */
apbf_status apbf_set_scene(apbf_ctx *ctx, const apbf_scene *scene);
/* Oriented boxes (no counterpart in the reference, whose boxes are axis-aligned):
 * appended after the boxes of the last apbf_set_boxes call, each given by its
 * centre, half extents (float4 each, w ignored) and rotation quaternion (x, y, z,
 * w; local -> world).  Box collision pushes a particle out of an oriented box with
 * the reference's rule (box_collision.comp:35-57) applied in the box's frame.
 * apbf_set_boxes removes them. */
apbf_status apbf_set_oriented_boxes(apbf_ctx *ctx, const float *center, const float *half, const float *quat,
                                    uint32_t n);
/* The rotation rows (3 float4 per box, the boxes' local axes; row 0 .w = 1 for an
 * oriented box, all zero for an axis-aligned one) of the first n boxes, as used on
 * the device. */
apbf_status apbf_get_box_rotations(apbf_ctx *ctx, float *rot_out, uint32_t n);
/* Particle emitter (no counterpart in the reference, whose scenes create all
 * particles up front): a lattice stream of spacing 2 radius, nx x nz cells wide,
 * moving at `speed` along -y through the emission plane y = origin[1].  Layer l
 * crosses the plane at t_l = l * 2 radius / speed; each apbf_substep(dt) first
 * appends the layers with T <= t_l < T + dt (T = stream time so far), at
 * y = origin[1] + (t_l - T) * speed (above the plane, so the substep's velocity
 * update carries them through it), x = origin[0] + (2i + 1) radius,
 * z = origin[2] + (2j + 1) radius, each coordinate jittered uniformly by up to
 * jitter * radius (hash of seed, layer, cell), velocity (0, -speed, 0) and the
 * fluid defaults of a particle of that radius.  Stops after max_particles (0: no
 * limit) or at the list capacity (APBF_FLAG_PARTICLE_OVERFLOW). */
typedef struct apbf_emitter {
    float origin[3];
    float radius;
    uint32_t nx, nz;
    float speed;
    float jitter;
    uint32_t seed;
    uint32_t max_particles;
    uint32_t enabled;
    uint32_t pad;
} apbf_emitter;
/* Sets the emitter and restarts its stream (T = 0, nothing emitted). */
apbf_status apbf_set_emitter(apbf_ctx *ctx, const apbf_emitter *e);
/* Axis-aligned collision boxes, vec4 min / vec4 max host arrays (user_controlled_boxes). */
apbf_status apbf_set_boxes(apbf_ctx *ctx, const float *box_min4, const float *box_max4, uint32_t n);

/* ---- list access (gpu_list::buffer / length, source/gpu_list.h) ---- */
apbf_status apbf_fluid_get_view(apbf_ctx *ctx, apbf_fluid_view *out);
/* Caller-owned lists, the reference's ownership model: its stages keep pointers to
 * lists the scene owns (neighborhood_green::set_data, neighborhood_green.h:11;
 * incompressibility::set_data, incompressibility.h:11; update_transfers::set_data,
 * update_transfers.h:11; particle_transfer::set_data, particle_transfer.h:11), and a
 * list edit moves a list to another of its pooled buffers (gpu_list.h:238-261).
 * apbf_bind_lists makes the context run every stage, apbf_substep and the host-list
 * copies on the caller's device memory: two buffer sets of the particle lists and
 * of the transfer list (a reorder, a compaction or a Jacobi pass writes one set from
 * the other), one length word per list (shared by its two sets), and the neighbour
 * rows (row_stride as apbf_neighbors_get_view reports it, at least max_neighbors
 * entries per row).  The context keeps only scratch (and the warm start's lambda
 * history); it allocates nothing in this call and never frees the caller's memory.
 * fluid[0] and transfers[0] are current at the bind; after any call
 * apbf_fluid_get_view / apbf_transfers_get_view name the caller's set that is
 * current, and the length words hold the lists' lengths (each stage call copies them
 * in before its work and out after it, stream-ordered).  int4 / float4 arrays must
 * be 16-byte aligned.  Synchronises the device; invalidates captured graphs. */
apbf_status apbf_bind_lists(apbf_ctx *ctx, const apbf_fluid_view fluid[2], const apbf_transfers_view transfers[2],
                            const apbf_neighbors_view *neighbors);
/* Back to the context's own lists, with the contents they had before the bind (set
 * their lengths, or upload, before the next stage call).  Synchronises the device. */
apbf_status apbf_unbind_lists(apbf_ctx *ctx);
apbf_status apbf_transfers_get_view(apbf_ctx *ctx, apbf_transfers_view *out);
apbf_status apbf_neighbors_get_view(apbf_ctx *ctx, apbf_neighbors_view *out);
/* The rows the position update gathers over besides the forward rows (no
 * reference counterpart: the reference scatters with atomics,
 * incompressibility_3.comp:62-66).  *union_rows (may be NULL; synchronises the
 * stream) receives 2 when every search radius was equal (the forward rows are
 * symmetric and serve alone; this view is unused), 1 for correction rows (the green
 * search with radii that differ: particle i's update sums over its forward row and
 * then over this row, whose entries with bit 31 set are entries j of i's forward
 * row whose own radius does not reach i, subtracted again, and whose other entries
 * are particles k whose forward rows hold i although i's radius does not reach k,
 * added), 0 for transposed rows (row j lists every i whose forward row holds j; the
 * forward rows are not used by the update). */
apbf_status apbf_neighbors_get_reverse_view(apbf_ctx *ctx, apbf_neighbors_view *out, uint32_t *union_rows,
                                            void *stream);
/* gpu_list::set_length with a host value (source/gpu_list.h:85-90). */
apbf_status apbf_set_lengths(apbf_ctx *ctx, uint32_t n_particles, uint32_t n_transfers, void *stream);
/* Reads the device lengths (synchronises the stream). */
apbf_status apbf_get_lengths(apbf_ctx *ctx, uint32_t *n_particles, uint32_t *n_transfers, void *stream);
/* gpu_list::write().buffer() filled from the host + set_length (source/gpu_list.h:82-91,
 * 173-180) for every particle list at once: enqueues the copies of `count` particles
 * from host memory and sets the particle length; nothing else of the state changes
 * (transfers, lambda history unless given).  Stream-ordered, no synchronisation.
 * Page-locked host arrays (cudaHostAlloc / cudaHostRegister) are read by one copy
 * kernel for all of them; pageable arrays are copied with cudaMemcpyAsync. */
apbf_status apbf_fluid_write(apbf_ctx *ctx, const apbf_host_fluid *in, uint32_t count, void *stream);
/* gpu_list::read (source/gpu_list.h:153-170) for every particle list at once: enqueues
 * the copy of the particle length into *h_count and of the first max_count entries of
 * every non-null field into host memory.  After the stream is synchronised, *h_count
 * is the number of particles (entries past min(*h_count, max_count) are not state).
 * Page-locked host arrays are written by one copy kernel for all of them. */
apbf_status apbf_fluid_read(apbf_ctx *ctx, apbf_host_fluid *out, uint32_t max_count, uint32_t *h_count, void *stream);

/* ---- stages (each replaces one reference stage's apply()) ---- */
/* velocity_handling::apply (source/velocity_handling.cpp:15-31). */
apbf_status apbf_velocity_handling_apply(apbf_ctx *ctx, float dt, const float acceleration[3], void *stream);
/* neighborhood_green::set_range_scale / set_position_range / apply
 * (source/neighborhood_green.h:11-14, source/neighborhood_green.cpp:27-77). */
apbf_status apbf_neighborhood_green_apply(apbf_ctx *ctx, float range_scale, const float min_pos[3],
                                          const float max_pos[3], uint32_t log2res, void *stream);
/* neighborhood_binary_search::set_range_scale / apply
 * (source/neighborhood_binary_search.h:11-12, source/neighborhood_binary_search.cpp:22-75):
 * sorts the particles by the 96-bit interleave of their raw coordinates and builds
 * each particle's row from the 27 cells of edge 2^k around its own cell, k the
 * smallest level with 2^k >= its search radius.  The rows hold the same neighbours
 * as apbf_neighborhood_green_apply's (the particle order differs); a row lists its
 * cells in the reference's order, x fastest, each cell in ascending index. */
apbf_status apbf_neighborhood_binary_search_apply(apbf_ctx *ctx, float range_scale, void *stream);
/* shader_provider::calculate_position_code (source/shader_provider.h:47,
 * calculate_position_code.comp:22-72): d_out[k] = 32-bit word code_section (0..2)
 * of the 96-bit code of particle d_index_list[k] (of particle k when d_index_list
 * is NULL), for every k below the particle count. */
apbf_status apbf_calculate_position_code(apbf_ctx *ctx, const uint32_t *d_index_list, uint32_t code_section,
                                         uint32_t *d_out, void *stream);
/* The neighbour search of apbf_substep, numbered as NEIGHBORHOOD_TYPE
 * (shaders/cpu_gpu_shared_config.h:5): Green (the default) or binary search. */
#define APBF_NEIGHBORHOOD_GREEN 1
#define APBF_NEIGHBORHOOD_BINARY_SEARCH 3
apbf_status apbf_set_neighborhood_search(apbf_ctx *ctx, int method);
/* box_collision::apply (source/box_collision.cpp:12-24). */
apbf_status apbf_box_collision_apply(apbf_ctx *ctx, void *stream);
/* incompressibility::apply, one Jacobi iteration (source/incompressibility.cpp:12-45). */
apbf_status apbf_incompressibility_apply(apbf_ctx *ctx, void *stream);
/* uint_to_float_with_indexed_lower_bound as called at source/pool.cpp:77-80. */
apbf_status apbf_kernel_width_from_boundary_distance_apply(apbf_ctx *ctx, void *stream);
/* spread_kernel_width::apply (source/spread_kernel_width.cpp:12-26). */
apbf_status apbf_spread_kernel_width_apply(apbf_ctx *ctx, void *stream);
/* update_transfers::apply (source/update_transfers.cpp:14-71). */
apbf_status apbf_update_transfers_apply(apbf_ctx *ctx, void *stream);
/* particle_transfer::apply (source/particle_transfer.cpp:10-28). */
apbf_status apbf_particle_transfer_apply(apbf_ctx *ctx, float dt, void *stream);
/* pool::update (source/pool.cpp:67-106): the whole substep with the scene set by
 * apbf_set_scene and the iteration count of the settings. */
apbf_status apbf_substep(apbf_ctx *ctx, float dt, void *stream);

/* ---- results and diagnostics ---- */
/* FP64 reductions into out[4] (host): total mass, total volume, mean compression
 * error max(0, rho/rho0 - 1) and mean |rho/rho0 - 1| of the last density pass.
 * No reference counterpart.  Synchronises the stream. */
apbf_status apbf_reduce_fp64(apbf_ctx *ctx, double out[4], void *stream);
/* Device status word (synchronises the stream); clears it when clear != 0. */
apbf_status apbf_get_status(apbf_ctx *ctx, apbf_status_info *out, int clear, void *stream);
/* The neighbour rows as the reference's uvec2 pair list (id, neighbour id); writes
 * min(pairs, capacity_pairs) pairs and the pair count to *d_length. */
apbf_status apbf_export_pairs(apbf_ctx *ctx, uint32_t *d_pairs, uint32_t capacity_pairs, uint32_t *d_length,
                              void *stream);
/* Enables (1) or disables (0) the capture of per-particle incompressibility
 * intermediates read by apbf_debug_incompressibility (costs 24 bytes per particle
 * of extra writes per iteration). */
apbf_status apbf_set_debug(apbf_ctx *ctx, int enable);
/* Bound of the context's device-side waits (no reference counterpart: the reference
 * has no cross-block waits): the decoupled look-backs of its sorts and scans and the
 * grid barriers of its persistent solves spin at most `limit` times (0: their
 * defaults, about 2^22) before giving up, setting APBF_FLAG_SPIN_LIMIT and returning,
 * so that apbf_get_status reports APBF_ERR_SPIN_LIMIT and the context stays usable.
 * inject != 0 makes every such wait treat the flag it waits for as never set, so each
 * wait runs out: a way to test the failure path without a fault or a hang.  Results
 * computed while a wait gave up are wrong (every index stays in bounds).  Synchronous;
 * not during stream capture. */
apbf_status apbf_set_wait_limit(apbf_ctx *ctx, uint32_t limit, int inject);
/* Graph use of apbf_substep (no counterpart in the reference):
 *   0  one launch per kernel, one launch pair per possible Jacobi pass;
 *   1  (default) Jacobi passes 1.. as one CUDA graph launch whose while loop ends
 *      on the device at convergence or after solver_iterations passes;
 *   2  the whole substep as one CUDA graph launch (captured on first use, one
 *      graph per buffer-role state and dt, replayed afterwards), the solve loop a
 *      conditional node inside it.
 * All modes give the same results.  Tracing, debugging and sample recording run
 * a substep with per-kernel launches. */
apbf_status apbf_set_solve_graph(apbf_ctx *ctx, int mode);
/* Jacobi passes 1.. of apbf_substep as one persistent cooperative kernel (no
 * counterpart in the reference): a resident grid runs every remaining pass, with
 * grid barriers between the density and position phases instead of two kernel
 * launches per pass.  Same results as the other forms.  Used for the Gauss kernels
 * without the centre-of-mass boundariness (method 1), outside tracing, debugging
 * and sample recording; otherwise apbf_set_solve_graph's form runs.  A barrier
 * wait that gives up sets the spin-limit status (APBF_ERR_SPIN_LIMIT).  Fails with
 * APBF_ERR_INVALID_ARG on a device without cooperative launches. */
apbf_status apbf_set_persistent_solve(apbf_ctx *ctx, int enable);

/* A batch of contexts (independent scenes on one device) advanced by one CUDA graph
 * launch per substep (apbf_batch_substep): every context's substep is a parallel
 * branch of the graph, each scene with its own solve loop and convergence.  The
 * contexts stay usable on their own; no context may be in two batches that run at
 * the same time.  No counterpart in the reference. */
typedef struct apbf_batch apbf_batch;
apbf_status apbf_batch_create(apbf_ctx *const *ctxs, uint32_t n, apbf_batch **out);
apbf_status apbf_batch_substep(apbf_batch *batch, float dt, void *stream);
apbf_status apbf_batch_destroy(apbf_batch *batch);
/* 1: the Jacobi passes 1.. of every context whose solve qualifies (see
 * apbf_set_persistent_solve) run as one persistent cooperative launch over a device
 * table of the scenes, between the branches' first passes and the rest of their
 * substeps (each scene keeps its own target, pass limit and convergence; results
 * bit-identical).  0 (default): each scene's solve loop stays in its branch, which
 * overlaps the scenes' loops instead of running every pass of every scene in
 * lockstep. */
apbf_status apbf_batch_set_persistent_solve(apbf_batch *batch, int enable);

/* Launch shapes (no counterpart in the reference).  apbf_autotune times every
 * candidate shape of the Jacobi passes on the context's current particle state and
 * neighbour rows (call it after a substep or a neighbourhood search), keeps the
 * fastest and restores the state it ran on; pass_ms (may be NULL) receives the
 * time of one pass for each of the 24 candidates, in the order gather_lanes
 * (1, 2, 4, 8) x pass_block (128, 256) x pass_blocks_per_sm (2, 4, 8). */
apbf_status apbf_set_tuning(apbf_ctx *ctx, const apbf_tuning *t);
apbf_status apbf_get_tuning(apbf_ctx *ctx, apbf_tuning *t);
apbf_status apbf_autotune(apbf_ctx *ctx, void *stream, apbf_tuning *chosen, float *pass_ms);
/* The neighbour search's tuning (no counterpart in the reference): times the radix
 * sort of apbf_substep's search for 6-, 7- and 8-bit digits, then the whole search
 * on grids of 2^(L-1), 2^L and 2^(L+1) cells per axis (L the current search grid;
 * only levels up to max_log2res), keeps the fastest digit width and grid in the
 * tuning (sort_digit_bits, search_log2res) and restores the particle state, the
 * transfer list and the status it ran on.  ms (may be NULL) receives six times:
 * the sort per digit width, the search per grid level (0 where not timed).  The
 * choice leaves the neighbour sets unchanged; the particle order follows the grid.
 * Not with a glue list. */
apbf_status apbf_autotune_search(apbf_ctx *ctx, void *stream, apbf_tuning *chosen, float *ms);
/* Per-particle intermediates of the last incompressibility iteration (debug):
 * density and squared-gradient sums (2^18 fixed point), weighted gradient sums
 * (int4), lambda.  Any pointer may be NULL. */
apbf_status apbf_debug_incompressibility(apbf_ctx *ctx, uint32_t *d_density, int32_t *d_grad_sum4,
                                         uint32_t *d_sq_grad_sum, float *d_lambda, void *stream);
/* Sort permutation (new id -> old id) and sorted cell keys of the last neighbourhood search. */
apbf_status apbf_debug_sort(apbf_ctx *ctx, uint32_t *d_perm, uint32_t *d_keys, void *stream);

/* ---- tracing (replaces measurements::record_timing_interval_*, source/measurements.cpp:27-62) ---- */
typedef struct apbf_kernel_time {
    char name[48];
    uint32_t launches;
    uint32_t pad;
    double total_ms; /* sum of CUDA-event durations on the launching stream */
} apbf_kernel_time;
/* Enables per-launch CUDA-event timing (capacity = events pairs kept until the
 * next apbf_profile_read; launches beyond it are counted as dropped). */
apbf_status apbf_profile_enable(apbf_ctx *ctx, int enable, uint32_t capacity);
/* Synchronises the stream, aggregates the recorded launches per kernel name into
 * out[0..*n_out) and clears the record. */
apbf_status apbf_profile_read(apbf_ctx *ctx, apbf_kernel_time *out, uint32_t cap, uint32_t *n_out,
                              unsigned long long *dropped, void *stream);
/* Number of kernels this context has launched since creation. */
apbf_status apbf_launch_count(apbf_ctx *ctx, unsigned long long *out);

/* ---- learned warm start of the Jacobi solve (no reference counterpart) ----
 * A 7 -> 64 -> 64 -> 1 ReLU network (BF16 weights, FP32 accumulation, tensor
 * cores) maps per-particle features of the first density pass of a substep --
 * neighbour count, rho/rho0 - 1, kernel width / radius, the plain Jacobi lambda,
 * velocity divergence / density, the sum of the lambdas applied to the particle
 * in the previous substep, and that sum's mean over the neighbours (8 slots, 7
 * used) -- to the lambda used by that substep's first position update.  Later
 * iterations are the plain solve, which still measures the density error and
 * stops at density_error_target.  Parameters are one FP32 vector of
 * apbf_mlp_param_count() floats: mu[8], 1/sigma[8], W1[64][8], b1[64],
 * W2[64][64], b2[64], w3[64], b3, y_scale, y_mean (lambda = y * y_scale + y_mean),
 * omega_max (> 0: the learned lambda is clamped to [omega_max * lambda, lambda]
 * where the plain lambda of the pass is negative and is 0 elsewhere),
 * min_neighbors (a particle with fewer neighbours keeps the plain lambda), three
 * reserved floats. */
apbf_status apbf_mlp_param_count(uint32_t *out);
/* Floats of scratch apbf_mlp_train_step needs for n_samples samples. */
apbf_status apbf_mlp_partials_size(uint32_t n_samples, uint32_t *out_floats);
/* Copies device parameters into the context. */
apbf_status apbf_mlp_load(apbf_ctx *ctx, const float *d_params, void *stream);
/* Warm-start mode of apbf_substep, a combination of:
 *   APBF_WARM_LEARNED    the first position update uses the network's lambda;
 *   APBF_WARM_PROJECTED  the later passes of the substep may apply a pull-back
 *                        (lambda > 0) up to the lambda sum the particle was pushed
 *                        with earlier in the substep, so an over-push is undone,
 *                        and the density that pull-back would restore counts in
 *                        the density error that density_error_target tests.
 * 0 is the reference's solve. */
#define APBF_WARM_LEARNED 1
#define APBF_WARM_PROJECTED 2
apbf_status apbf_set_warm_start(apbf_ctx *ctx, int mode);
/* Arms the next apbf_substep to append one training sample per particle: its 8
 * features (first density pass) and the sum of min(0, lambda) over the first
 * `iterations` plain Jacobi iterations; d_count (device) is advanced, at most
 * `capacity` samples are kept. */
apbf_status apbf_record_samples(apbf_ctx *ctx, uint32_t iterations, float *d_features, float *d_targets,
                                uint32_t capacity, uint32_t *d_count);
/* Inference on n feature rows (8 floats each): d_out = lambda in physical units. */
apbf_status apbf_mlp_forward(const float *d_params, const float *d_features, uint32_t n, float *d_out, void *stream);
/* One Adam step (lr; step = number of earlier steps) on the weighted mean squared
 * error between the normalised output y and d_targets t (already normalised):
 * mean of w (y - t)^2 with w = over_weight (> 0) where y < t -- a larger push than
 * the target -- and 1 elsewhere (over_weight = 1: plain least squares).
 * d_partials holds apbf_mlp_partials_size(n) floats; d_grad (may be NULL)
 * receives the gradient, d_loss (may be NULL) the loss.  lr = 0 leaves the
 * parameters and moments unchanged. */
apbf_status apbf_mlp_train_step(float *d_params, float *d_m, float *d_v, float *d_partials, const float *d_features,
                                const float *d_targets, uint32_t n, float lr, float over_weight, uint32_t step,
                                float *d_grad, float *d_loss, void *stream);

/* ---- further constraint operators on the same lists ---- */
/* sphere_collision::apply (source/sphere_collision.cpp:19-31, sphere_collision.comp):
 * hollow != 0 keeps the particles inside the sphere, 0 outside. */
apbf_status apbf_sphere_collision_apply(apbf_ctx *ctx, const float center[3], float radius, int hollow, void *stream);
/* inter_particle_collision::apply (source/inter_particle_collision.cpp:10-18): one
 * Jacobi step of the non-penetration constraint over the pairs of the neighbour
 * rows of the last search. */
apbf_status apbf_inter_particle_collision_apply(apbf_ctx *ctx, void *stream);
/* glue::applyNewGlue (source/glue.cpp:48-60): replaces the glue list by the pairs of
 * the neighbour rows that generate_glue.comp glues, in row order (the reference
 * appends them unordered); grows the list to `capacity` entries on demand
 * (APBF_FLAG_TRANSFER_OVERFLOW when more pairs qualify).  Glue ids follow later
 * neighbour-search reorders. */
apbf_status apbf_glue_generate(apbf_ctx *ctx, uint32_t capacity, void *stream);
/* glue::apply (source/glue.cpp:38-46, glue.comp), every entry reading the positions
 * before the pass (glue.comp reads the buffer it updates, a race). */
apbf_status apbf_glue_apply(apbf_ctx *ctx, float stability, float elasticity, void *stream);
/* The glue list: particle ids, rest distances (2^18 fixed point), device length. */
apbf_status apbf_glue_get_view(apbf_ctx *ctx, uint32_t **p0, uint32_t **p1, uint32_t **dist, uint32_t **d_length,
                               uint32_t *capacity);

/* save_particle_info::apply (source/save_particle_info.cpp:22-125): writes
 * centerDist.txt, radius.txt, neighborCount.txt, kernelWidth.txt, targetRadius.txt,
 * boundaryDistance.txt (';'-separated) and data.csv (sorted by the distance to
 * `center`, stably) into `folder`, with the reference's formatting; the
 * reference's centre is (0, 10, -60).  Synchronises the stream. */
apbf_status apbf_save_particle_info(apbf_ctx *ctx, const char *folder, const float center[3], void *stream);

/* ---- list-edit services (gpu_list / indexed_list, source/gpu_list.h, indexed_list.h) ----
 * On plain device arrays with device lengths; the context provides scratch (its
 * particle capacity bounds the lengths).  Results are deterministic. */
/* gpu_list::apply_edit (gpu_list.h:125-135, copy_scattered_read.comp): dst[k] =
 * src[edit[k]], stride_words 32-bit words per element, min(*d_edit_len, max_edit)
 * elements (d_edit_len may be NULL: max_edit). */
apbf_status apbf_list_apply_edit(const uint32_t *d_src, uint32_t stride_words, const uint32_t *d_edit,
                                 const uint32_t *d_edit_len, uint32_t max_edit, uint32_t *d_dst, void *stream);
/* indexed_list::delete_these (indexed_list.h:125-138): the edit list keeping every
 * hidden id in [0, n_hidden) not named in d_deleted, in increasing order. */
apbf_status apbf_list_delete_edit(apbf_ctx *ctx, const uint32_t *d_deleted, const uint32_t *d_deleted_len,
                                  uint32_t max_deleted, uint32_t n_hidden, uint32_t *d_edit, uint32_t *d_edit_len,
                                  void *stream);
/* indexed_list::apply_hidden_edit (indexed_list.h:288-308): the index list after its
 * hidden list was rebuilt by `edit` (new id e takes old id edit[e]): one entry e per
 * old entry equal to edit[e], ordered by e, then by old position; d_new_edit (may be
 * NULL) receives each entry's old position.  At most out_cap entries; d_required
 * (may be NULL) receives the full count.  A duplication is the edit [0, n) followed
 * by the duplicated ids (indexed_list::duplicate_these, indexed_list.h:140-152). */
apbf_status apbf_list_remap_index(apbf_ctx *ctx, const uint32_t *d_list, const uint32_t *d_list_len,
                                  uint32_t max_list, const uint32_t *d_edit, const uint32_t *d_edit_len,
                                  uint32_t max_edit, uint32_t n_hidden_old, uint32_t *d_out, uint32_t *d_new_edit,
                                  uint32_t out_cap, uint32_t *d_out_len, uint32_t *d_required, void *stream);
/* gpu_list::operator+= (gpu_list.h:213-227, append_list.comp): appends src to dst up
 * to dst_cap elements; d_scratch_word is one device word. */
apbf_status apbf_list_append(uint32_t *d_dst, uint32_t *d_dst_len, uint32_t dst_cap, const uint32_t *d_src,
                             const uint32_t *d_src_len, uint32_t max_src, uint32_t stride_words,
                             uint32_t *d_scratch_word, void *stream);

/* ---- parallel primitives (source/algorithms.h:12-17) ---- */
/* algorithms::sort (source/algorithms.cpp:59-91): stable sort of (key, value) pairs
 * by key; only key bits below the highest set bit of value_upper_bound are used.
 * n is read from d_count; max_count bounds it. */
apbf_status apbf_sort_pairs(apbf_ctx *ctx, const uint32_t *d_keys, const uint32_t *d_values, const uint32_t *d_count,
                            uint32_t max_count, uint32_t value_upper_bound, uint32_t *d_out_keys,
                            uint32_t *d_out_values, void *stream);
/* The same stable sort as apbf_sort_pairs, but it allocates nothing and needs no
 * context.  It has no counterpart in the reference.  It is meant for callers that
 * cannot call cudaMalloc: hosts whose device memory is owned by another allocator,
 * and per-frame code on which cudaMalloc / cudaFree would synchronise the device.
 * Its scratch is one fixed array in the library's device memory, held on every
 * device that loads the library until the process exits; max_count above
 * 1048576 (1 << 20) is rejected with APBF_ERR_INVALID_ARG, as are outputs that
 * overlap an input or each other (each buffer taken as max_count words).  The
 * first call on a device looks up that array's address on the current device and
 * keeps it for the life of the process; make that first call before any stream
 * capture, and do not use the entry point after cudaDeviceReset in the same
 * process (the module may then be loaded at another address).  All calls share
 * the array: calls whose work overlaps on the GPU (other streams, other threads)
 * race and must be serialised by the caller.  A bounded look-back wait that gives
 * up (which does not happen in normal operation) leaves the output out of order
 * and cannot be detected by the caller. */
apbf_status apbf_sort_pairs_noalloc(const uint32_t *d_keys, const uint32_t *d_values, const uint32_t *d_count,
                                    uint32_t max_count, uint32_t value_upper_bound, uint32_t *d_out_keys,
                                    uint32_t *d_out_values, void *stream);
/* algorithms::prefix_sum (source/algorithms.cpp:93-101): inclusive scan in place. */
apbf_status apbf_prefix_sum(apbf_ctx *ctx, uint32_t *d_values, const uint32_t *d_count, uint32_t max_count,
                            void *stream);

#ifdef __cplusplus
}
#endif
#endif
