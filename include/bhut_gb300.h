/*
 * bhut_gb300.h -- C ABI of the GB300 Barnes-Hut engine (libbhut_gb300.so).
 *
 * A drop-in for the compute behind bhut 0.1.0's public API
 * (bhut/api.py: accelerations, Tree.build/refit/rebuild/accelerations).
 * Plain pointers and sizes only.  Every array pointer may be host memory or
 * device memory of the current CUDA device (detected per call); arrays are
 * C-ordered float64 (positions (n, dim), masses (n,), accelerations
 * (n, dim)).  Calls are synchronous: outputs are complete on return.
 * Every call returns a status code (BHUT_OK == 0); bhut_last_error() gives the
 * message of the last failure on the calling thread.  Kernels never trap: a
 * device-side problem sets an error word that the call turns into
 * BHUT_EDEVICE.
 *
 * Handles are not thread-safe for concurrent mutation (as the reference's
 * Tree); concurrent calls on different handles are fine.
 */
#ifndef BHUT_GB300_H
#define BHUT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define BHUT_API __attribute__((visibility("default")))
#else
#define BHUT_API
#endif

#define BHUT_OK 0
#define BHUT_EINVAL 1      /* invalid argument (ValueError in the reference) */
#define BHUT_ENOTBUILT 2   /* tree not built */
#define BHUT_ECUDA 3       /* CUDA runtime failure */
#define BHUT_ENOMEM 4      /* device allocation failed */
#define BHUT_EDEVICE 5     /* a kernel reported an error (e.g. stack overflow) */
#define BHUT_EINTERNAL 6

/* Traversal arithmetic (bhut_tree_set_form). */
#define BHUT_FORM_EXACT 0  /* FP64; pair terms bit-identical to the reference's Numba loop */
#define BHUT_FORM_FAST 1   /* FP64-accurate float-float on the FP32 pipe (default) */
#define BHUT_FORM_FP32 2   /* precision form: FP32 with Kahan-compensated sums */

/* Opening criteria (bhut_tree_set_criterion). */
#define BHUT_MAC_BH 0      /* 2 h / |x - com| >= theta -> open (bhut/traverse/bh.py:576-601) */
#define BHUT_MAC_OFFSET 1  /* open when |x - com| < 2 h / theta + |com - AABB centre| */

/* Node expansions (bhut_tree_set_multipole, bhut_batch_set_multipole). */
#define BHUT_MULTIPOLE_MONO 0  /* monopole (bhut/traverse/kernels.py:136-168) */
#define BHUT_MULTIPOLE_QUAD 1  /* monopole + traceless quadrupole, FP32 form only */

typedef struct bhut_tree bhut_tree;

/* Library version string. */
BHUT_API const char *bhut_version(void);

/* Copies the last error message of this thread into buf (NUL-terminated);
 * returns its full length. */
BHUT_API int bhut_last_error(char *buf, size_t len);

/* New, unbuilt tree handle.  Replaces Tree.__init__ (bhut/api.py:470-495)
 * minus the array validation that the host layer does.  stream: a
 * cudaStream_t, or NULL for a stream owned by the handle. */
BHUT_API int bhut_tree_create(int dim, int leaf_size, void *stream, bhut_tree **out);

/* Builds the tree over n particles.  Replaces build_tree
 * (bhut/api.py:155-191 -> bhut/tree/build.py:19-107): bounding box, Morton
 * keys, stable sort, count-split topology, node AABBs, masses, COMs.
 * BHUT_EINVAL for n == 0 ("Cannot build tree with zero particles") or
 * non-finite positions. */
BHUT_API int bhut_tree_build(bhut_tree *t, const double *positions, const double *masses, int64_t n);

/* Tree.refit (bhut/api.py:513-562): when any particle lies outside 1.1x the
 * root box (bhut/tree/refit.py:195-251) or n differs, rebuilds and sets
 * *rebuilt = 1; else refit_tree (bhut/tree/refit.py:17-109) with stale node
 * geometry and permutation.  masses == NULL keeps the stored masses. */
BHUT_API int bhut_tree_refit(bhut_tree *t, const double *positions, const double *masses, int64_t n,
                    int *rebuilt);

/* Tree.rebuild (bhut/api.py:564-606).  masses == NULL keeps the stored
 * masses (n must then equal the stored n). */
BHUT_API int bhut_tree_rebuild(bhut_tree *t, const double *positions, const double *masses, int64_t n);

/* Self accelerations of the stored particles, out (n, dim).  Replaces
 * barnes_hut_accelerations (bhut/traverse/bh.py:428-548). */
BHUT_API int bhut_tree_accel_self(bhut_tree *t, double theta, double softening, double G, double *out);

/* Accelerations at m external targets (m, dim), out (m, dim).  Replaces
 * barnes_hut_accelerations_targets (bhut/traverse/bh.py:30-146). */
BHUT_API int bhut_tree_accel_targets(bhut_tree *t, const double *targets, int64_t m, double theta,
                            double softening, double G, double *out);

/* Selects the traversal arithmetic (BHUT_FORM_*). */
BHUT_API int bhut_tree_set_form(bhut_tree *t, int form);

/* Interaction counts of the last traversal on this handle: pair (P2P)
 * evaluations, monopole (M2P) evaluations and node visits, summed over
 * targets.  The device-side counterpart of compute_tree_statistics
 * (bhut/traverse/bh.py:604-700), counting pairs actually evaluated (the
 * target itself and zero-distance pairs are not counted). */
BHUT_API int bhut_tree_stats(const bhut_tree *t, int64_t *p2p, int64_t *m2p, int64_t *visits);

/* Fallbacks of the last fast-form traversal: opening decisions that fell in
 * the FP32 test's error band and were taken by the exact FP64 test, and
 * pairs evaluated in FP64 (closer than 2^-15 of the box half-size). */
BHUT_API int bhut_tree_fallbacks(const bhut_tree *t, int64_t *exact_decisions, int64_t *fp64_pairs);

/* Total number of kernels this library has launched in the process. */
BHUT_API long long bhut_launch_count(void);

/* Opening criterion of the FP32 form (BHUT_MAC_*; default BHUT_MAC_BH).  The
 * exact and fast forms always use the reference criterion.  No counterpart
 * in the reference, whose only criterion is "bh" (bhut/api.py:306-307). */
BHUT_API int bhut_tree_set_criterion(bhut_tree *t, int criterion);

/* Node expansion of the FP32 form (BHUT_MULTIPOLE_*; default monopole).  The
 * exact and fast forms always use monopoles.  No counterpart in the
 * reference, whose only multipole is "mono" (bhut/api.py:308-309). */
BHUT_API int bhut_tree_set_multipole(bhut_tree *t, int multipole);

/* n, node count, dim, leaf size of a built tree. */
BHUT_API int bhut_tree_info(const bhut_tree *t, int64_t *n, int64_t *num_nodes, int *dim, int *leaf_size);

/* Copies the TreeData arrays (bhut/tree/node.py:15-77) to host buffers sized
 * for num_nodes (center and com: num_nodes x dim) and n (perm).  Any pointer
 * may be NULL to skip that array. */
BHUT_API int bhut_tree_export(const bhut_tree *t, double *center, double *half_size, double *mass,
                     double *com, int64_t *first_child, int64_t *child_count, int64_t *start,
                     int64_t *count, uint8_t *is_leaf, int64_t *perm);

/* Releases the handle and its device memory. */
BHUT_API void bhut_tree_destroy(bhut_tree *t);

/* Morton keys in input order: aabb + normalize_to_unit + morton_codes
 * (bhut/space/bbox.py:14-96, bhut/utils/morton.py:48-102). */
BHUT_API int bhut_morton_keys(const double *positions, int64_t n, int dim, uint64_t *keys, void *stream);

/* sort_by_morton (bhut/utils/morton.py:105-147): sorted keys and the stable
 * permutation (np.argsort(kind='stable')). */
BHUT_API int bhut_morton_argsort(const double *positions, int64_t n, int dim, uint64_t *sorted_keys,
                        int64_t *perm, void *stream);

/* Morton keys + stable argsort that allocates no device memory.  No
 * counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc (GPU memory owned by another allocator, or a step loop where an
 * allocation would synchronize the device).  Same result as
 * bhut_morton_argsort, with perm as int32.  All pointers must be memory of
 * the current device (or managed memory); n <= 1,048,576.  Scratch is one
 * static device array (about 13.7 MB, held on every GPU that loads the
 * library until exit) shared by all calls: calls that overlap on the GPU
 * race.  The first call on a device looks up the array's address; make it
 * before any stream capture, and make no call after cudaDeviceReset.  Each
 * call reads its error word back and synchronizes its stream before it
 * returns. */
BHUT_API int bhut_morton_argsort_noalloc(const double *positions, int64_t n, int dim,
                                         uint64_t *sorted_keys, int32_t *perm, void *stream);

/* ---- batched form: many independent systems per solve ------------------ */
/* No counterpart in the reference (which solves one system per call); each
 * system's result equals a single-system solve with the same form.  Systems
 * are concatenated: positions (N_total, dim), masses (N_total,), system s
 * owns particles [offsets[s], offsets[s+1]). */
typedef struct bhut_batch bhut_batch;

BHUT_API int bhut_batch_create(int dim, int leaf_size, void *stream, bhut_batch **out);

/* form: BHUT_FORM_FP32 (default) or BHUT_FORM_FAST; criterion: BHUT_MAC_*;
 * targets_per_warp: 32 or 16 (two lanes per target); use_graph: capture the
 * whole solve (build + traversal) in a CUDA graph and replay it while the
 * layout, theta, softening, G and output buffer stay the same. */
BHUT_API int bhut_batch_configure(bhut_batch *b, int form, int criterion, int targets_per_warp,
                                  int use_graph);

/* Placement of the batched traversal's per-warp stack (bhut_batch_set_stack):
 * shared memory, or registers spread over the warp's lanes (two entries per
 * lane, popped with shuffles).  A tuning choice; results are identical. */
#define BHUT_STACK_SHARED 0
#define BHUT_STACK_REGISTERS 1
BHUT_API int bhut_batch_set_stack(bhut_batch *b, int placement);

/* Node expansion of the batched FP32 form (BHUT_MULTIPOLE_*; default
 * monopole); no counterpart in the reference. */
BHUT_API int bhut_batch_set_multipole(bhut_batch *b, int multipole);

/* Copies the systems in; a new layout (offsets) re-plans node counts, buffers
 * and the task queue. */
BHUT_API int bhut_batch_load(bhut_batch *b, const double *positions, const double *masses,
                             const int64_t *offsets, int64_t nsys);

/* Builds every tree and evaluates all self accelerations; out (N_total, dim)
 * in input order. */
BHUT_API int bhut_batch_solve(bhut_batch *b, double theta, double softening, double G, double *out);

BHUT_API int bhut_batch_info(const bhut_batch *b, int64_t *nsys, int64_t *n_total,
                             int64_t *nodes_total, int64_t *tasks);

/* Pair, monopole and node-visit counts of the last solve. */
BHUT_API int bhut_batch_stats(const bhut_batch *b, int64_t *p2p, int64_t *m2p, int64_t *visits);

/* Refit instead of rebuild for chosen systems: for every s with keep[s] != 0
 * the next solves reuse the Morton order of `perm` (global indices, the
 * layout of the last load) instead of sorting; node boxes, masses and
 * centres of mass are recomputed from the current positions, the topology
 * is unchanged.  keep == NULL returns to a full rebuild of every system. */
BHUT_API int bhut_batch_keep_order(bhut_batch *b, const uint8_t *keep, const int32_t *perm);

/* Copies the permutation of the last solve (global indices) to perm; stream
 * ordered (no host synchronisation) when perm is device memory. */
BHUT_API int bhut_batch_order(const bhut_batch *b, int32_t *perm);

/* The refit-vs-rebuild test inside the solve (on: 1): a system asked to keep
 * its order (bhut_batch_keep_order) is rebuilt instead when a particle lies
 * beyond 1.1 x its stored root box (bhut/tree/refit.py:236-249); every
 * rebuilt system's root box is stored.  Roots and counts of forced rebuilds
 * are per system of the current layout (zeroed by a new layout). */
BHUT_API int bhut_batch_set_refit_rule(bhut_batch *b, int on);
BHUT_API int bhut_batch_set_roots(bhut_batch *b, const double *roots);
BHUT_API int bhut_batch_forced(const bhut_batch *b, int32_t *counts);

/* Root centre (3 doubles, zero-padded in 2-D) and half-size of every system,
 * 4 doubles per system (host or device pointer): the stored roots with the
 * refit rule on, else those of the last solve. */
BHUT_API int bhut_batch_roots(const bhut_batch *b, double *roots);

/* should_refit_vs_rebuild (bhut/tree/refit.py:236-249) for every system of
 * the loaded positions against the given roots (4 doubles per system):
 * flags[s] = 1 when system s must be rebuilt. */
BHUT_API int bhut_batch_outside(const bhut_batch *b, const double *roots, uint8_t *flags);

BHUT_API void bhut_batch_destroy(bhut_batch *b);

/* Device time of the traversal kernel of the last solve (CUDA events
 * recorded around it, also inside a replayed graph), in milliseconds.  No
 * counterpart in the reference; used for the roofline of the batched form. */
BHUT_API int bhut_batch_traverse_ms(const bhut_batch *b, double *ms);

/* Leapfrog update on device arrays (n, dim): v += kick * a, then, when
 * drift != 0, x += drift * v.  A kick-drift-kick step is
 * (kick = dt/2, drift = dt), a new acceleration, then (kick = dt/2, drift = 0). */
BHUT_API int bhut_leapfrog(double *positions, double *velocities, const double *accelerations,
                           int64_t n, int dim, double kick, double drift, void *stream);

/* FP64 direct sum (the theta = 0 limit) at m targets, or self accelerations
 * when targets == NULL (then m must equal n). */
BHUT_API int bhut_direct_accelerations(const double *positions, const double *masses, int64_t n, int dim,
                              const double *targets, int64_t m, double softening, double G,
                              double *out, void *stream);

/* Operation counts of compute_tree_statistics (bhut/traverse/bh.py:604-700)
 * for any TreeData arrays (host or device pointers; int64 indices, com as
 * (num_nodes, dim)): totals[0] = nodes visited, totals[1] = particles
 * computed, totals[2] = monopoles used, summed over the nt targets (the
 * reference divides by the target count for its averages). */
BHUT_API int bhut_tree_statistics(const double *com, const double *half_size, const double *mass,
                                  const int64_t *first_child, const int64_t *child_count,
                                  const int64_t *start, const int64_t *count, int64_t num_nodes,
                                  int dim, const double *targets, int64_t nt, double theta,
                                  void *stream, int64_t *totals);

/* ---- module-level stages (host or device pointers; synchronous) ---------- */

/* aabb (bhut/space/bbox.py:14-46): per-axis min and max of n points.
 * NaN propagates as in numpy.  dim 1..3. */
BHUT_API int bhut_aabb(const double *points, int64_t n, int dim, double *pmin, double *pmax,
                       void *stream);

/* normalize_to_unit (bhut/space/bbox.py:49-96): (x - pmin) / extent + offset,
 * degenerate axes mapped to 0.5, clamped at 1 - eps.  pmin, pmax: host
 * arrays of dim doubles. */
BHUT_API int bhut_normalize_to_unit(const double *points, int64_t n, int dim, const double *pmin,
                                    const double *pmax, double eps, double *out, void *stream);

/* morton_codes (bhut/utils/morton.py:48-102) of points already in [0, 1)^dim,
 * `bits` per axis (1..62); BHUT_EINVAL "All points must be in range [0, 1)"
 * otherwise. */
BHUT_API int bhut_morton_codes_unit(const double *points01, int64_t n, int dim, int bits,
                                    uint64_t *codes, void *stream);

/* sort_by_morton (bhut/utils/morton.py:105-147): codes of points01, stably
 * sorted; perm (int64) = original index of each sorted point. */
BHUT_API int bhut_sort_morton_unit(const double *points01, int64_t n, int dim, int bits,
                                   uint64_t *sorted_codes, int64_t *perm, void *stream);

/* dst[i] = src[perm[i]] for n rows of row_bytes bytes (the data_arrays of
 * sort_by_morton, bhut/utils/morton.py:139-145). */
BHUT_API int bhut_gather_rows(const void *src, int64_t n, int64_t row_bytes, const int64_t *perm,
                              void *dst, void *stream);

/* should_refit_vs_rebuild (bhut/tree/refit.py:195-251) boundary test: *refit
 * = 0 when any point lies beyond 1.1 x root_half from root_center along
 * some axis, else 1. */
BHUT_API int bhut_should_refit(const double *positions, int64_t n, int dim,
                               const double *root_center, double root_half, int *refit,
                               void *stream);

/* refit_tree (bhut/tree/refit.py:17-109) alone: new leaf and internal masses
 * and centres of mass through the frozen permutation, geometry kept, no
 * refit-vs-rebuild test (bhut_tree_refit adds that test and the rebuild). */
BHUT_API int bhut_tree_refit_only(bhut_tree *t, const double *positions, const double *masses,
                                  int64_t n);

/* Loads a TreeData built elsewhere (bhut/tree/node.py:15-77; int64 indices,
 * com and center as (num_nodes, dim)) with the particles it indexes, so
 * that bhut_tree_accel_self / accel_targets / refit / export run on it
 * (barnes_hut_accelerations bhut/traverse/bh.py:428-482, refit_tree
 * bhut/tree/refit.py:17-109).  Binary trees only (child_count 0 or 2). */
BHUT_API int bhut_tree_import(bhut_tree *t, const double *positions, const double *masses,
                              int64_t n, const int64_t *first_child, const int64_t *child_count,
                              const int64_t *start, const int64_t *count, const int64_t *perm,
                              const double *center, const double *half_size, const double *mass,
                              const double *com, int64_t num_nodes);

/* Measured FP32 FMA peak of the current GPU (TFLOP/s): independent FMA
 * chains on every SM, best of 2 timed runs.  A measurement utility for the
 * FP32-pipe rooflines; no reference counterpart. */
BHUT_API int bhut_measure_fp32_peak(double *tflops);

/* Bytes in use and reserved by the stream-ordered pool that holds the
 * engine's device buffers (current device). */
BHUT_API int bhut_pool_usage(int64_t *used, int64_t *reserved);

/* Returns the pool's reserved but unused device memory to the driver
 * (synchronises the device); the server calls it after retiring requests. */
BHUT_API int bhut_pool_trim(void);

#ifdef __cplusplus
}
#endif

#endif /* BHUT_GB300_H */
