/*
 * bhut_oracle.c -- CPU restatement of the bhut 0.1.0 hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the CUDA engine in
 * bhut_gb300/csrc is checked against.  Only tests/, the smoke check in
 * __graft_entry__.py and the CPU-baseline / reference arm of bench.py may
 * load it.  The product path never calls it and has no CPU fallback.
 *
 * Parity is pinned: tests/golden/make_golden.py imports the reference
 * package, runs it on seeded inputs and stores its outputs; the CPU test
 * suite checks this restatement against those fixtures (keys, perm, tree
 * arrays bit-exact, accelerations to 1e-12 relative).
 *
 * Every function names the reference file:line it restates.  All arithmetic
 * is scalar IEEE binary64; compile with -ffp-contract=off so that no fused
 * multiply-add changes a rounding (the reference's Numba loop is not fused).
 *
 * Two numpy primitives carry arithmetic that the reference depends on:
 *  - numpy (2.x) 1-D float64 np.sum uses pairwise summation
 *    (numpy/_core/src/umath/loops_utils.h.src, pairwise_sum): blocks of at
 *    most 128 elements summed with 8 interleaved accumulators, larger ranges
 *    split at n/2 rounded down to a multiple of 8.  np.sum(axis=0) of an
 *    (n, D) C-ordered array is a plain row-order sequential sum.
 *  - np.linalg.norm of a 3-vector is sqrt(x.dot(x)); on x86-64 the bundled
 *    OpenBLAS ddot tail loop is a fused multiply-add chain,
 *    fma(z, z, fma(y, y, x*x)).
 * Both facts were checked bit-for-bit against numpy in this container; they
 * are restated in pairwise_sum() and should_open() below.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define EXPORT __attribute__((visibility("default")))

/* ------------------------------------------------------------------------ */
/* numpy pairwise sum (np.sum of a contiguous 1-D float64 array)            */
/* ------------------------------------------------------------------------ */
static double pairwise_sum(const double *a, int64_t n)
{
    if (n < 8) {
        double res = -0.0;
        for (int64_t i = 0; i < n; i++) res += a[i];
        return res;
    } else if (n <= 128) {
        double r[8];
        for (int j = 0; j < 8; j++) r[j] = a[j];
        int64_t i;
        for (i = 8; i < n - (n % 8); i += 8)
            for (int j = 0; j < 8; j++) r[j] += a[i + j];
        double res = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
        for (; i < n; i++) res += a[i];
        return res;
    } else {
        int64_t n2 = n / 2;
        n2 -= n2 % 8;
        return pairwise_sum(a, n2) + pairwise_sum(a + n2, n - n2);
    }
}

/* np.sum(x) for a 1-D array: the reduction starts from the additive
 * identity and adds the pairwise sum of all elements. */
static double np_sum(const double *a, int64_t n) { return 0.0 + pairwise_sum(a, n); }

/* ------------------------------------------------------------------------ */
/* bbox.py:14-46 aabb, bbox.py:49-96 normalize_to_unit,                      */
/* morton.py:14-102 morton_codes, morton.py:105-147 sort_by_morton           */
/* ------------------------------------------------------------------------ */
EXPORT void bo_aabb(const double *pos, int64_t n, int dim, double *pmin, double *pmax)
{
    for (int d = 0; d < dim; d++) {
        double lo = pos[d], hi = pos[d];
        for (int64_t i = 1; i < n; i++) {
            double v = pos[i * dim + d];
            if (v < lo) lo = v;
            if (v > hi) hi = v;
        }
        pmin[d] = lo;
        pmax[d] = hi;
    }
}

static uint64_t expand_bits_3d(uint64_t x)      /* morton.py:31-45 */
{
    x = (x | (x << 32)) & 0x1F00000000FFFFull;
    x = (x | (x << 16)) & 0x1F0000FF0000FFull;
    x = (x | (x << 8)) & 0x100F00F00F00F00Full;
    x = (x | (x << 4)) & 0x10C30C30C30C30C3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

static uint64_t expand_bits_2d(uint64_t x)      /* morton.py:14-28 */
{
    x = (x | (x << 16)) & 0x0000FFFF0000FFFFull;
    x = (x | (x << 8)) & 0x00FF00FF00FF00FFull;
    x = (x | (x << 4)) & 0x0F0F0F0F0F0F0F0Full;
    x = (x | (x << 2)) & 0x3333333333333333ull;
    x = (x | (x << 1)) & 0x5555555555555555ull;
    return x;
}

/* Morton key of every particle, in input order.  Quantisation follows
 * bbox.py:85-94 (degenerate axis -> extent 1, offset 0.5; clamp 1-1e-12)
 * and morton.py:183-198 (truncate p01 * 2^21, clamp to 2^21-1). */
EXPORT void bo_morton(const double *pos, int64_t n, int dim, const double *pmin,
                      const double *pmax, uint64_t *codes)
{
    const double top = 1.0 - 1e-12;
    const double scale = (double)(1u << 21);
    const uint64_t max_coord = (1u << 21) - 1;
    double extent[3], offset[3];
    for (int d = 0; d < dim; d++) {
        double e = pmax[d] - pmin[d];
        extent[d] = (e <= 0) ? 1.0 : e;
        offset[d] = (e <= 0) ? 0.5 : 0.0;
    }
    for (int64_t i = 0; i < n; i++) {
        uint64_t c[3];
        for (int d = 0; d < dim; d++) {
            double p = (pos[i * dim + d] - pmin[d]) / extent[d] + offset[d];
            if (p > top) p = top;          /* np.minimum(points01, 1 - eps) */
            uint64_t q = (uint64_t)(p * scale);
            c[d] = q < max_coord ? q : max_coord;
        }
        if (dim == 3)
            codes[i] = expand_bits_3d(c[0]) | (expand_bits_3d(c[1]) << 1) | (expand_bits_3d(c[2]) << 2);
        else
            codes[i] = expand_bits_2d(c[0]) | (expand_bits_2d(c[1]) << 1);
    }
}

/* Stable argsort of uint64 keys (np.argsort(kind='stable'), morton.py:135).
 * A stable order is unique, so any stable method gives the same perm; this
 * one is an LSD radix sort with 8-bit digits. */
EXPORT void bo_stable_argsort(const uint64_t *keys, int64_t n, int64_t *perm)
{
    int64_t *tmp = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    for (int64_t i = 0; i < n; i++) perm[i] = i;
    int64_t *src = perm, *dst = tmp;
    for (int pass = 0; pass < 8; pass++) {
        int shift = pass * 8;
        int64_t cnt[257];
        memset(cnt, 0, sizeof(cnt));
        for (int64_t i = 0; i < n; i++) cnt[((keys[src[i]] >> shift) & 0xFF) + 1]++;
        for (int b = 0; b < 256; b++) cnt[b + 1] += cnt[b];
        for (int64_t i = 0; i < n; i++) dst[cnt[(keys[src[i]] >> shift) & 0xFF]++] = src[i];
        int64_t *t = src; src = dst; dst = t;
    }
    /* eight passes: the result is back in perm */
    free(tmp);
}

/* ------------------------------------------------------------------------ */
/* build.py:110-212 _build_tree_iterative                                    */
/* ------------------------------------------------------------------------ */
EXPORT int64_t bo_max_nodes(int64_t n, int leaf_size)
{
    int64_t m = 4 * n / leaf_size;      /* build.py:124 */
    return m > 10 ? m : 10;
}

/* Count-median binary split with node ids handed out in pop order of a LIFO
 * stack (left child pushed first, so the right child is processed first).
 * Returns the node count, or -1 when max_nodes would be exceeded (the
 * reference's out-of-space fallback at build.py:166-169 is unreachable). */
EXPORT int64_t bo_topology(int64_t n, int leaf_size, int64_t max_nodes,
                           int64_t *first_child, int64_t *child_count,
                           int64_t *start, int64_t *count, uint8_t *is_leaf)
{
    for (int64_t i = 0; i < max_nodes; i++) {
        first_child[i] = -1; child_count[i] = 0; start[i] = 0; count[i] = 0; is_leaf[i] = 0;
    }
    int64_t cap = 128, sp = 0;
    int64_t *stack = (int64_t *)malloc(sizeof(int64_t) * 3 * (size_t)cap);
    stack[0] = 0; stack[1] = 0; stack[2] = n; sp = 1;
    int64_t node_count = 1;
    while (sp > 0) {
        sp--;
        int64_t node = stack[3 * sp], s = stack[3 * sp + 1], e = stack[3 * sp + 2];
        int64_t c = e - s;
        if (node >= max_nodes) { free(stack); return -1; }
        start[node] = s;
        count[node] = c;
        if (c <= leaf_size) {
            is_leaf[node] = 1;
            continue;
        }
        if (node_count + 2 > max_nodes) { free(stack); return -1; }
        int64_t mid = s + c / 2;
        first_child[node] = node_count;
        child_count[node] = 2;
        if (sp + 2 > cap) {
            cap *= 2;
            stack = (int64_t *)realloc(stack, sizeof(int64_t) * 3 * (size_t)cap);
        }
        /* left (start, mid) pushed first, right (mid, end) second */
        if (s < mid) { stack[3 * sp] = node_count; stack[3 * sp + 1] = s; stack[3 * sp + 2] = mid; sp++; }
        if (mid < e) { stack[3 * sp] = node_count + 1; stack[3 * sp + 1] = mid; stack[3 * sp + 2] = e; sp++; }
        node_count += 2;
    }
    free(stack);
    return node_count;
}

/* build.py:215-242 _compute_node_geometry: tight AABB of each node's sorted
 * particles; the root uses the global pmin/pmax (same values). */
EXPORT void bo_geometry(const double *spos, int dim, int64_t num_nodes, const int64_t *start,
                        const int64_t *count, const double *pmin, const double *pmax,
                        double *center, double *half_size)
{
    for (int64_t k = 0; k < num_nodes; k++) {
        double lo[3] = {0.0, 0.0, 0.0}, hi[3] = {0.0, 0.0, 0.0};
        if (k == 0) {
            for (int d = 0; d < dim; d++) { lo[d] = pmin[d]; hi[d] = pmax[d]; }
        } else {
            int64_t s = start[k], c = count[k];
            if (c <= 0) { for (int d = 0; d < dim; d++) center[k * dim + d] = 0.0; half_size[k] = 0.0; continue; }
            for (int d = 0; d < dim; d++) { lo[d] = spos[s * dim + d]; hi[d] = lo[d]; }
            for (int64_t i = s + 1; i < s + c; i++)
                for (int d = 0; d < dim; d++) {
                    double v = spos[i * dim + d];
                    if (v < lo[d]) lo[d] = v;
                    if (v > hi[d]) hi[d] = v;
                }
        }
        double ext_max = hi[0] - lo[0];
        for (int d = 0; d < dim; d++) {
            center[k * dim + d] = (lo[d] + hi[d]) / 2;
            double e = hi[d] - lo[d];
            if (e > ext_max) ext_max = e;
        }
        half_size[k] = ext_max / 2;
    }
}

/* Leaf mass and centre of mass from the particles listed by idx[0..c):
 * build.py:259-271 and refit.py:133-149 (both gather into a contiguous
 * array, np.sum it pairwise, and sum m_i * x_i row by row). */
static void leaf_moments(const double *pos, const double *m, const int64_t *idx, int64_t c,
                         int dim, const double *center, double *mass_out, double *com_out,
                         double *scratch)
{
    for (int64_t i = 0; i < c; i++) scratch[i] = m[idx[i]];
    double total = np_sum(scratch, c);
    *mass_out = total;
    if (total > 0) {
        double acc[3] = {0.0, 0.0, 0.0};
        for (int64_t i = 0; i < c; i++)
            for (int d = 0; d < dim; d++) acc[d] = acc[d] + scratch[i] * pos[idx[i] * dim + d];
        for (int d = 0; d < dim; d++) com_out[d] = acc[d] / total;
    } else {
        for (int d = 0; d < dim; d++) com_out[d] = center[d];
    }
}

/* build.py:245-295 _compute_mass_and_com (reverse node order; children have
 * larger ids than parents).  spos/smass are the Morton-sorted arrays. */
EXPORT void bo_mass_com(const double *spos, const double *smass, int dim, int64_t num_nodes,
                        const int64_t *first_child, const int64_t *child_count,
                        const int64_t *start, const int64_t *count, const uint8_t *is_leaf,
                        const double *center, double *mass, double *com)
{
    int64_t maxc = 1;
    for (int64_t k = 0; k < num_nodes; k++) if (is_leaf[k] && count[k] > maxc) maxc = count[k];
    double *scratch = (double *)malloc(sizeof(double) * (size_t)maxc);
    int64_t *idx = (int64_t *)malloc(sizeof(int64_t) * (size_t)maxc);
    for (int64_t k = num_nodes - 1; k >= 0; k--) {
        if (is_leaf[k]) {
            int64_t s = start[k], c = count[k];
            if (c > 0) {
                for (int64_t i = 0; i < c; i++) idx[i] = s + i;
                leaf_moments(spos, smass, idx, c, dim, center + k * dim, &mass[k], com + k * dim, scratch);
            } else {
                mass[k] = 0.0;
                for (int d = 0; d < dim; d++) com[k * dim + d] = center[k * dim + d];
            }
        } else {
            int64_t f = first_child[k], nc = child_count[k];
            if (nc > 0) {
                double cm[8];
                for (int64_t j = 0; j < nc; j++) cm[j] = mass[f + j];
                double total = np_sum(cm, nc);
                if (total > 0) {
                    double acc[3] = {0.0, 0.0, 0.0};
                    for (int64_t j = 0; j < nc; j++)
                        for (int d = 0; d < dim; d++) acc[d] = acc[d] + cm[j] * com[(f + j) * dim + d];
                    for (int d = 0; d < dim; d++) com[k * dim + d] = acc[d] / total;
                } else {
                    for (int d = 0; d < dim; d++) com[k * dim + d] = center[k * dim + d];
                }
                mass[k] = total;
            } else {
                mass[k] = 0.0;
                for (int d = 0; d < dim; d++) com[k * dim + d] = center[k * dim + d];
            }
        }
    }
    free(scratch);
    free(idx);
}

/* Full build_tree (build.py:19-107).  Arrays are sized for max_nodes
 * (bo_max_nodes); returns the node count or a negative error. */
EXPORT int64_t bo_build(const double *pos, const double *m, int64_t n, int dim, int leaf_size,
                        uint64_t *codes, int64_t *perm, double *center, double *half_size,
                        double *mass, double *com, int64_t *first_child, int64_t *child_count,
                        int64_t *start, int64_t *count, uint8_t *is_leaf)
{
    if (n <= 0) return -2;
    double pmin[3], pmax[3];
    bo_aabb(pos, n, dim, pmin, pmax);
    bo_morton(pos, n, dim, pmin, pmax, codes);
    bo_stable_argsort(codes, n, perm);
    double *spos = (double *)malloc(sizeof(double) * (size_t)(n * dim));
    double *smass = (double *)malloc(sizeof(double) * (size_t)n);
    for (int64_t i = 0; i < n; i++) {
        for (int d = 0; d < dim; d++) spos[i * dim + d] = pos[perm[i] * dim + d];
        smass[i] = m[perm[i]];
    }
    int64_t max_nodes = bo_max_nodes(n, leaf_size);
    int64_t nn = bo_topology(n, leaf_size, max_nodes, first_child, child_count, start, count, is_leaf);
    if (nn < 0) { free(spos); free(smass); return -3; }
    for (int64_t k = 0; k < nn * dim; k++) { center[k] = 0.0; com[k] = 0.0; }
    for (int64_t k = 0; k < nn; k++) { half_size[k] = 0.0; mass[k] = 0.0; }
    bo_geometry(spos, dim, nn, start, count, pmin, pmax, center, half_size);
    bo_mass_com(spos, smass, dim, nn, first_child, child_count, start, count, is_leaf, center, mass, com);
    free(spos);
    free(smass);
    return nn;
}

/* ------------------------------------------------------------------------ */
/* refit.py:17-192 refit_tree; refit.py:195-251 should_refit_vs_rebuild      */
/* ------------------------------------------------------------------------ */
EXPORT void bo_refit(const double *pos, const double *m, int dim, int64_t num_nodes,
                     const int64_t *first_child, const int64_t *child_count,
                     const int64_t *start, const int64_t *count, const uint8_t *is_leaf,
                     const int64_t *perm, const double *center, double *mass, double *com)
{
    int64_t maxc = 1;
    for (int64_t k = 0; k < num_nodes; k++) if (is_leaf[k] && count[k] > maxc) maxc = count[k];
    double *scratch = (double *)malloc(sizeof(double) * (size_t)maxc);
    /* refit.py:112-149: leaves, in node order, particles via perm */
    for (int64_t k = 0; k < num_nodes; k++) {
        if (!is_leaf[k]) continue;
        if (count[k] == 0) {
            mass[k] = 0.0;
            for (int d = 0; d < dim; d++) com[k * dim + d] = 0.0;
            continue;
        }
        leaf_moments(pos, m, perm + start[k], count[k], dim, center + k * dim, &mass[k],
                     com + k * dim, scratch);
    }
    /* refit.py:152-192: internal nodes in reverse order; children whose mass
     * is not positive are skipped (unlike the build) */
    for (int64_t k = num_nodes - 1; k >= 0; k--) {
        if (is_leaf[k]) continue;
        int64_t f = first_child[k], nc = child_count[k];
        if (f == -1 || nc == 0) {
            mass[k] = 0.0;
            for (int d = 0; d < dim; d++) com[k * dim + d] = center[k * dim + d];
            continue;
        }
        double total = 0.0, w[3] = {0.0, 0.0, 0.0};
        for (int64_t j = 0; j < nc; j++) {
            int64_t ch = f + j;
            if (ch >= num_nodes) break;
            double cmass = mass[ch];
            if (cmass > 0) {
                total += cmass;
                for (int d = 0; d < dim; d++) w[d] = w[d] + cmass * com[ch * dim + d];
            }
        }
        mass[k] = total;
        if (total > 0)
            for (int d = 0; d < dim; d++) com[k * dim + d] = w[d] / total;
        else
            for (int d = 0; d < dim; d++) com[k * dim + d] = center[k * dim + d];
    }
    free(scratch);
}

EXPORT int bo_should_refit(const double *root_center, double root_half, const double *pos,
                           int64_t n, int dim)
{
    double lim = 1.1 * root_half;
    for (int64_t i = 0; i < n; i++) {
        double mx = fabs(pos[i * dim] - root_center[0]);
        for (int d = 1; d < dim; d++) {
            double v = fabs(pos[i * dim + d] - root_center[d]);
            if (v > mx) mx = v;
        }
        if (mx > lim) return 0;
    }
    return 1;
}

/* ------------------------------------------------------------------------ */
/* Traversal: bh.py:485-548 (self) and bh.py:83-146 (external targets)       */
/* ------------------------------------------------------------------------ */

/* bh.py:576-601 _should_open_node: d = ||x - com|| (numpy norm: FMA chain
 * through OpenBLAS ddot on x86-64), open when d == 0 or 2h/d >= theta. */
static int should_open(const double *x, const double *c, double size, double theta, int dim)
{
    double s;
    if (dim == 3) {
        double dx = x[0] - c[0], dy = x[1] - c[1], dz = x[2] - c[2];
        s = fma(dz, dz, fma(dy, dy, dx * dx));
    } else {
        double dx = x[0] - c[0], dy = x[1] - c[1];
        s = fma(dy, dy, dx * dx);
    }
    double d = sqrt(s);
    if (d == 0) return 1;
    return (size / d) >= theta;
}

/* kernels.py:14-95 acc_monopole (single vector) via acc_monopole_node
 * kernels.py:136-168: dx = com - x, r2 = sum(dx^2) + eps^2,
 * a = (G*M) / r2^1.5 * dx, zero when r2 == 0. */
static void monopole(const double *x, const double *c, double M, double eps, double G,
                     int dim, double *out)
{
    double dx[3], r2 = -0.0;
    for (int d = 0; d < dim; d++) { dx[d] = c[d] - x[d]; r2 += dx[d] * dx[d]; }
    r2 = 0.0 + r2;
    double r2s = r2 + eps * eps;
    if (r2s == 0) { for (int d = 0; d < dim; d++) out[d] = 0.0; return; }
    double f = (G * M) / pow(r2s, 1.5);
    for (int d = 0; d < dim; d++) out[d] = f * dx[d];
}

/* bh.py:226-280 _numba_leaf_particle_loop (self_idx >= 0 skips the target
 * itself) and bh.py:173-223 (external, self_idx < 0).  A pair with
 * r^2 + eps^2 == 0 contributes nothing: Numba raises ZeroDivisionError there
 * and the reference falls back to the pure-Python loop (bh.py:339-343,
 * 384-425), whose kernel returns zero for that pair (kernels.py:62-63). */
static void leaf_p2p(const double *x, int64_t self_idx, const double *pos, const double *m,
                     const int64_t *perm, int64_t s, int64_t c, double eps, double G, int dim,
                     double *out, int64_t *n_p2p)
{
    double acc[3] = {0.0, 0.0, 0.0};
    double eps2 = eps * eps;
    for (int64_t i = s; i < s + c; i++) {
        int64_t p = perm[i];
        if (p == self_idx) continue;
        double dx[3], r2 = 0.0;
        for (int d = 0; d < dim; d++) { dx[d] = pos[p * dim + d] - x[d]; r2 += dx[d] * dx[d]; }
        r2 += eps2;
        if (r2 == 0) continue;
        double r = sqrt(r2);
        double ri = 1.0 / r;
        double ri3 = ri * ri * ri;
        double f = G * m[p] * ri3;
        for (int d = 0; d < dim; d++) acc[d] += f * dx[d];
        (*n_p2p)++;
    }
    for (int d = 0; d < dim; d++) out[d] = acc[d];
}

typedef struct {
    const double *com, *half_size, *mass;
    const int64_t *first_child, *child_count, *start, *count, *perm;
    int64_t num_nodes;
} tree_view;

static void traverse_one(const tree_view *t, const double *pos, const double *m, const double *x,
                         int64_t self_idx, double theta, double eps, double G, int dim,
                         double *out, int64_t *stats)
{
    double acc[3] = {0.0, 0.0, 0.0}, part[3];
    int64_t stack[512];
    int sp = 0;
    stack[sp++] = 0;
    int64_t visits = 0, mono = 0, p2p = 0;
    while (sp > 0) {
        int64_t k = stack[--sp];
        visits++;
        if (k < 0 || k >= t->num_nodes) continue;
        if (t->mass[k] == 0) continue;
        if (t->first_child[k] == -1) {
            if (t->count[k] <= 0) continue;
            leaf_p2p(x, self_idx, pos, m, t->perm, t->start[k], t->count[k], eps, G, dim, part, &p2p);
            for (int d = 0; d < dim; d++) acc[d] += part[d];
        } else if (should_open(x, t->com + k * dim, 2 * t->half_size[k], theta, dim)) {
            int64_t ch = t->first_child[k];
            for (int64_t j = 0; j < t->child_count[k]; j++) {
                if (sp >= 512) { out[0] = out[1] = out[2] = NAN; return; }
                stack[sp++] = ch + j;
            }
        } else {
            monopole(x, t->com + k * dim, t->mass[k], eps, G, dim, part);
            for (int d = 0; d < dim; d++) acc[d] += part[d];
            mono++;
        }
    }
    for (int d = 0; d < dim; d++) out[d] = acc[d];
    if (stats) { stats[0] = visits; stats[1] = p2p; stats[2] = mono; }
}

/* Accelerations at nt targets.  self_idx == NULL: external targets
 * (bh.py:30-80); otherwise target i is source particle self_idx[i]
 * (bh.py:428-482, evaluated for any subset of particles).  stats, when not
 * NULL, receives per-target (node visits, P2P pairs, monopoles). */
EXPORT void bo_accel(const double *com, const double *half_size, const double *mass,
                     const int64_t *first_child, const int64_t *child_count,
                     const int64_t *start, const int64_t *count, const int64_t *perm,
                     int64_t num_nodes, const double *pos, const double *m, int dim,
                     const double *targets, int64_t nt, const int64_t *self_idx,
                     double theta, double eps, double G, double *out, int64_t *stats,
                     int nthreads)
{
    tree_view t = {com, half_size, mass, first_child, child_count, start, count, perm, num_nodes};
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
#endif
    for (int64_t i = 0; i < nt; i++) {
        const double *x = self_idx ? pos + self_idx[i] * dim : targets + i * dim;
        traverse_one(&t, pos, m, x, self_idx ? self_idx[i] : -1, theta, eps, G, dim,
                     out + i * dim, stats ? stats + 3 * i : NULL);
    }
    (void)nthreads;
}

/* Operation counts of compute_tree_statistics (bh.py:604-700): for each
 * target, the nodes popped (empty and out-of-range ones included), the
 * particles of every visited non-empty leaf minus one (count - 1, whether or
 * not the target lies in that leaf) and the accepted internal nodes, with the
 * opening test of bh.py:576-601.  totals = (nodes_visited,
 * particles_computed, monopoles_used) summed over the targets. */
EXPORT int bo_tree_statistics(const double *com, const double *half_size, const double *mass,
                              const int64_t *first_child, const int64_t *child_count,
                              const int64_t *start, const int64_t *count, int64_t num_nodes,
                              int dim, const double *targets, int64_t nt, double theta,
                              int64_t *totals, int nthreads)
{
    int64_t nodes = 0, parts = 0, monos = 0;
    int bad = 0;
    (void)nthreads;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads) \
    reduction(+ : nodes, parts, monos, bad)
#endif
    for (int64_t i = 0; i < nt; i++) {
        const double *x = targets + i * dim;
        int64_t stack[512];
        int sp = 0;
        stack[sp++] = 0;
        while (sp > 0) {
            int64_t k = stack[--sp];
            nodes++;
            if (k < 0 || k >= num_nodes || mass[k] == 0) continue;
            if (first_child[k] == -1) {
                if (start[k] != -1 && count[k] > 0) parts += count[k] - 1;
            } else if (should_open(x, com + k * dim, 2 * half_size[k], theta, dim)) {
                int64_t ch = first_child[k];
                for (int64_t j = 0; j < child_count[k]; j++) {
                    if (sp >= 512) { bad++; sp = 0; break; }
                    stack[sp++] = ch + j;
                }
            } else {
                monos++;
            }
        }
    }
    totals[0] = nodes;
    totals[1] = parts;
    totals[2] = monos;
    return bad ? -1 : 0;
}

/* FP64 direct sum over all sources (the theta = 0 limit, bh.py:226-280
 * arithmetic).  self_idx as in bo_accel. */
EXPORT void bo_direct(const double *pos, const double *m, int64_t n, int dim,
                      const double *targets, int64_t nt, const int64_t *self_idx,
                      double eps, double G, double *out, int nthreads)
{
    (void)nthreads;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
#endif
    for (int64_t i = 0; i < nt; i++) {
        const double *x = self_idx ? pos + self_idx[i] * dim : targets + i * dim;
        int64_t me = self_idx ? self_idx[i] : -1;
        double acc[3] = {0.0, 0.0, 0.0};
        double eps2 = eps * eps;
        for (int64_t p = 0; p < n; p++) {
            if (p == me) continue;
            double dx[3], r2 = 0.0;
            for (int d = 0; d < dim; d++) { dx[d] = pos[p * dim + d] - x[d]; r2 += dx[d] * dx[d]; }
            r2 += eps2;
            if (r2 == 0) continue;
            double ri = 1.0 / sqrt(r2);
            double f = G * m[p] * (ri * ri * ri);
            for (int d = 0; d < dim; d++) acc[d] += f * dx[d];
        }
        for (int d = 0; d < dim; d++) out[i * dim + d] = acc[d];
    }
}

EXPORT int bo_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
