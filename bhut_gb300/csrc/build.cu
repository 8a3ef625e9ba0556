// Tree construction and refit kernels.
//
//   K1 k_bbox            FP64 AABB of the input      bhut/space/bbox.py:14-46
//   K2 k_morton          normalise + Morton key      bhut/space/bbox.py:49-96,
//                                                    bhut/utils/morton.py:14-102
//   K3 radix_sort_pairs  stable argsort (sort.cu)    bhut/utils/morton.py:105-147
//   K4 k_gather_sorted   sorted SoA + perm           bhut/tree/build.py:89-92
//   K5 k_topology        count-split tree            bhut/tree/build.py:110-212
//   K6 k_bottom_up       AABB, mass, COM per node    bhut/tree/build.py:215-295
//                        (refit mode)                bhut/tree/refit.py:17-192
//   k_outside_root       refit-vs-rebuild test       bhut/tree/refit.py:195-251
//
// Everything that the reference computes bit-exactly (keys, permutation,
// topology, node AABBs, masses and centres of mass) is reproduced
// bit-exactly: the arithmetic uses explicit round-to-nearest intrinsics so
// nvcc cannot contract a multiply and an add, and the summation orders match
// numpy's (pairwise for a 1-D np.sum, row order for np.sum(axis=0)).
#include <cstdarg>
#include <cstdio>
#include "tree.cuh"

namespace bhut {

// ---------------------------------------------------------------------------
// K1: bounding box.  Block partials, the last block to finish reduces them
// (no waiting: a block that is not last just exits).
// ---------------------------------------------------------------------------
constexpr int kBoxThreads = 256;

__global__ void __launch_bounds__(kBoxThreads)
k_bbox(const double* __restrict__ pos, const double* __restrict__ mass, int64_t n, int dim,
       double* __restrict__ partial, unsigned* __restrict__ done_counter, double* __restrict__ box,
       unsigned* __restrict__ err)
{
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    double mmax = 0.0;
    bool bad = false;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        for (int d = 0; d < dim; d++) {
            double v = pos[i * dim + d];
            bad |= !isfinite(v);
            lo[d] = v < lo[d] ? v : lo[d];
            hi[d] = v > hi[d] ? v : hi[d];
        }
        if (mass) {
            double am = fabs(mass[i]);
            bad |= !isfinite(am);
            mmax = am > mmax ? am : mmax;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        double a = __shfl_down_sync(0xffffffffu, mmax, o);
        mmax = a > mmax ? a : mmax;
    }
    __shared__ double s_m[kBoxThreads / 32];
    if ((threadIdx.x & 31) == 0) s_m[threadIdx.x >> 5] = mmax;
    __shared__ double s_lo[3][kBoxThreads / 32], s_hi[3][kBoxThreads / 32];
    __shared__ bool s_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int d = 0; d < 3; d++) {
        for (int o = 16; o > 0; o >>= 1) {
            double a = __shfl_down_sync(0xffffffffu, lo[d], o);
            double b = __shfl_down_sync(0xffffffffu, hi[d], o);
            lo[d] = a < lo[d] ? a : lo[d];
            hi[d] = b > hi[d] ? b : hi[d];
        }
        if (lane == 0) { s_lo[d][warp] = lo[d]; s_hi[d][warp] = hi[d]; }
    }
    if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(err, kErrNonFinite);
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int d = 0; d < 3; d++) {
            double a = s_lo[d][0], b = s_hi[d][0];
            for (int w = 1; w < kBoxThreads / 32; w++) {
                a = s_lo[d][w] < a ? s_lo[d][w] : a;
                b = s_hi[d][w] > b ? s_hi[d][w] : b;
            }
            partial[blockIdx.x * 8 + d] = a;
            partial[blockIdx.x * 8 + 3 + d] = b;
        }
        double mm = s_m[0];
        for (int w = 1; w < kBoxThreads / 32; w++) mm = s_m[w] > mm ? s_m[w] : mm;
        partial[blockIdx.x * 8 + 6] = mm;
        __threadfence();
        unsigned ticket = atomicAdd(done_counter, 1u);
        s_last = (ticket == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return;
    // last block: reduce all partials in parallel (strided over blocks)
    __threadfence();
    double a[7];
    for (int d = 0; d < 3; d++) { a[d] = INFINITY; a[3 + d] = -INFINITY; }
    a[6] = 0.0;
    for (unsigned g = threadIdx.x; g < gridDim.x; g += blockDim.x) {
        for (int d = 0; d < 3; d++) {
            double x = __ldcg(&partial[g * 8 + d]), y = __ldcg(&partial[g * 8 + 3 + d]);
            a[d] = x < a[d] ? x : a[d];
            a[3 + d] = y > a[3 + d] ? y : a[3 + d];
        }
        double mm = __ldcg(&partial[g * 8 + 6]);
        a[6] = mm > a[6] ? mm : a[6];
    }
    for (int o = 16; o > 0; o >>= 1) {
        for (int d = 0; d < 3; d++) {
            double x = __shfl_down_sync(0xffffffffu, a[d], o);
            double y = __shfl_down_sync(0xffffffffu, a[3 + d], o);
            a[d] = x < a[d] ? x : a[d];
            a[3 + d] = y > a[3 + d] ? y : a[3 + d];
        }
        double mm = __shfl_down_sync(0xffffffffu, a[6], o);
        a[6] = mm > a[6] ? mm : a[6];
    }
    __shared__ double s_fin[kBoxThreads / 32][7];
    if (lane == 0)
        for (int k = 0; k < 7; k++) s_fin[warp][k] = a[k];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kBoxThreads / 32; w++) {
            for (int d = 0; d < 3; d++) {
                a[d] = s_fin[w][d] < a[d] ? s_fin[w][d] : a[d];
                a[3 + d] = s_fin[w][3 + d] > a[3 + d] ? s_fin[w][3 + d] : a[3 + d];
            }
            a[6] = s_fin[w][6] > a[6] ? s_fin[w][6] : a[6];
        }
        for (int k = 0; k < 7; k++) box[k] = a[k];
        *done_counter = 0;
    }
}

// ---------------------------------------------------------------------------
// K2: Morton keys (input order) and the identity payload for the sort.
// ---------------------------------------------------------------------------
__global__ void k_morton(const double* __restrict__ pos, int64_t n, int dim,
                         const double* __restrict__ box, uint64_t* __restrict__ keys,
                         int32_t* __restrict__ idx)
{
    double pmin[3], ext[3], off[3];
    for (int d = 0; d < dim; d++) {
        pmin[d] = box[d];
        double e = __dsub_rn(box[3 + d], box[d]);
        ext[d] = e <= 0 ? 1.0 : e;
        off[d] = e <= 0 ? 0.5 : 0.0;
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t key;
        if (dim == 3) {
            key = morton3(quantise(pos[3 * i], pmin[0], ext[0], off[0]),
                          quantise(pos[3 * i + 1], pmin[1], ext[1], off[1]),
                          quantise(pos[3 * i + 2], pmin[2], ext[2], off[2]));
        } else {
            key = morton2(quantise(pos[2 * i], pmin[0], ext[0], off[0]),
                          quantise(pos[2 * i + 1], pmin[1], ext[1], off[1]));
        }
        keys[i] = key;
        if (idx) idx[i] = (int32_t)i;
    }
}

// ---------------------------------------------------------------------------
// K4: Morton-ordered SoA copy of positions and masses.
// ---------------------------------------------------------------------------
__global__ void k_gather_sorted(const double* __restrict__ pos, const double* __restrict__ mass,
                                const int32_t* __restrict__ perm, int64_t n, int dim,
                                double* __restrict__ sx, double* __restrict__ sy,
                                double* __restrict__ sz, double* __restrict__ sm)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        int64_t p = perm[i];
        sx[i] = pos[p * dim];
        sy[i] = pos[p * dim + 1];
        sz[i] = dim == 3 ? pos[p * dim + 2] : 0.0;
        if (mass) sm[i] = mass[p];
    }
}

// ---------------------------------------------------------------------------
// K5: topology.  One thread per BFS slot (depth d, index j): the path bits of
// j pick left/right halves from the root.  A node's id follows from the
// internal-node rank k of its parent (children 2k+1, 2k+2) and the ranks
// follow the right-first preorder of the reference's LIFO build stack: the
// right child of internal node k has rank k+1, the left child has rank
// k + 1 + (internal nodes in the right subtree).
// ---------------------------------------------------------------------------
__global__ void k_topology(TopoTables tt, int32_t* __restrict__ first_child,
                           int32_t* __restrict__ start, int32_t* __restrict__ count,
                           int32_t* __restrict__ parent, int32_t* __restrict__ leaf_list,
                           unsigned* __restrict__ leaf_counter, unsigned* __restrict__ err)
{
    const int64_t L = tt.leaf_size;
    for (int64_t slot = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; slot < tt.slots;
         slot += (int64_t)gridDim.x * blockDim.x) {
        int d = 63 - __clzll((unsigned long long)(slot + 1));   // depth
        int64_t j = slot + 1 - (1ll << d);                       // index in level
        int64_t c = tt.n, s = 0, k = 0, id = 0, par = -1;
        bool exists = true;
        for (int t = 0; t < d; t++) {
            if (c <= L) { exists = false; break; }
            int bit = (int)((j >> (d - 1 - t)) & 1);
            int64_t half = c / 2;
            int64_t rc = c - half;
            par = id;
            if (bit == 0) {
                id = 2 * k + 1;
                int64_t lo = tt.cnt_lo[t + 1];
                int64_t irc = tt.internal[t + 1][rc - lo];
                k = k + 1 + irc;
                c = half;
            } else {
                id = 2 * k + 2;
                k = k + 1;
                s += half;
                c = rc;
            }
        }
        if (!exists) continue;
        if (id >= tt.num_nodes || s + c > tt.n) { atomicOr(err, kErrBadNode); continue; }
        start[id] = (int32_t)s;
        count[id] = (int32_t)c;
        parent[id] = (int32_t)par;
        if (c <= L) {
            first_child[id] = -1;
            unsigned li = atomicAdd(leaf_counter, 1u);
            if (li < tt.num_leaves) leaf_list[li] = (int32_t)id;
            else atomicOr(err, kErrBadNode);
        } else {
            first_child[id] = (int32_t)(2 * k + 1);
        }
    }
}

// ---------------------------------------------------------------------------
// K6: bottom-up pass with per-node arrival counters.  A leaf thread computes
// its leaf, then climbs: the first child to arrive at a parent stops, the
// second computes the parent (both children are complete by then).  Parents
// always combine left then right, so the result does not depend on arrival
// order.
// ---------------------------------------------------------------------------
// numpy pairwise summation of a contiguous float64 block (n <= 128):
// eight interleaved accumulators, combined ((r0+r1)+(r2+r3))+((r4+r5)+(r6+r7)).
template <class F>
__device__ double pw_block(F load, int64_t base, int64_t n)
{
    if (n < 8) {
        double r = -0.0;
        for (int64_t i = 0; i < n; i++) r = __dadd_rn(r, load(base + i));
        return r;
    }
    double r[8];
#pragma unroll
    for (int j = 0; j < 8; j++) r[j] = load(base + j);
    int64_t i = 8;
    for (; i < n - (n % 8); i += 8) {
#pragma unroll
        for (int j = 0; j < 8; j++) r[j] = __dadd_rn(r[j], load(base + i + j));
    }
    double res = __dadd_rn(__dadd_rn(__dadd_rn(r[0], r[1]), __dadd_rn(r[2], r[3])),
                           __dadd_rn(__dadd_rn(r[4], r[5]), __dadd_rn(r[6], r[7])));
    for (; i < n; i++) res = __dadd_rn(res, load(base + i));
    return res;
}

// Full pairwise sum: ranges above 128 split at n/2 rounded down to a
// multiple of 8, left half summed before the right, evaluated with an
// explicit stack (post-order).
template <class F>
__device__ double pairwise_sum(F load, int64_t n)
{
    if (n <= 128) return pw_block(load, 0, n);
    struct Frame { int64_t base, n; int state; double left; };
    Frame st[48];
    int sp = 0;
    st[sp++] = {0, n, 0, 0.0};
    double ret = 0.0;
    while (sp > 0) {
        Frame& f = st[sp - 1];
        if (f.n <= 128) { ret = pw_block(load, f.base, f.n); sp--; continue; }
        int64_t n2 = f.n / 2;
        n2 -= n2 % 8;
        if (f.state == 0) { f.state = 1; st[sp++] = {f.base, n2, 0, 0.0}; }
        else if (f.state == 1) { f.left = ret; f.state = 2; st[sp++] = {f.base + n2, f.n - n2, 0, 0.0}; }
        else { ret = __dadd_rn(f.left, ret); sp--; }
    }
    return ret;
}

// One leaf: tight AABB (build only), pairwise mass, row-order weighted sum.
// In refit mode positions come from the caller's original-order arrays via
// perm (refit.py:133-149); in build mode from the sorted SoA.
__device__ void leaf_node(int32_t id, int dim, bool refit, const TreeDev& t,
                          const double* __restrict__ opos, const double* __restrict__ omass,
                          const int32_t* __restrict__ start, const int32_t* __restrict__ count,
                          NodeOut o)
{
    const int64_t s = start[id], c = count[id];
    double total;
    double acc[3] = {0.0, 0.0, 0.0};
    if (!refit) {
        auto ld = [&](int64_t i) { return t.sm[s + i]; };
        total = __dadd_rn(0.0, pairwise_sum(ld, c));
        double lo[3], hi[3];
        const double* axes[3] = {t.sx, t.sy, t.sz};
        for (int d = 0; d < dim; d++) { lo[d] = axes[d][s]; hi[d] = lo[d]; }
        for (int64_t i = 0; i < c; i++) {
            double mi = t.sm[s + i];
            for (int d = 0; d < dim; d++) {
                double v = axes[d][s + i];
                lo[d] = v < lo[d] ? v : lo[d];
                hi[d] = v > hi[d] ? v : hi[d];
                acc[d] = __dadd_rn(acc[d], __dmul_rn(mi, v));
            }
        }
        double ext = 0.0;
        for (int d = 0; d < dim; d++) {
            o.lo[3 * id + d] = lo[d];
            o.hi[3 * id + d] = hi[d];
            o.center[dim * id + d] = __dmul_rn(__dadd_rn(lo[d], hi[d]), 0.5);
            double e = __dsub_rn(hi[d], lo[d]);
            ext = (d == 0 || e > ext) ? e : ext;
        }
        o.half[id] = __dmul_rn(ext, 0.5);
        o.size[id] = __dmul_rn(2.0, o.half[id]);
    } else {
        auto ld = [&](int64_t i) { return omass[t.perm[s + i]]; };
        total = __dadd_rn(0.0, pairwise_sum(ld, c));
        for (int64_t i = 0; i < c; i++) {
            int64_t p = t.perm[s + i];
            double mi = omass[p];
            for (int d = 0; d < dim; d++)
                acc[d] = __dadd_rn(acc[d], __dmul_rn(mi, opos[p * dim + d]));
        }
    }
    NodeCM cm;
    double com[3];
    for (int d = 0; d < 3; d++) com[d] = 0.0;
    if (total > 0) {
        for (int d = 0; d < dim; d++) com[d] = __ddiv_rn(acc[d], total);
    } else {
        for (int d = 0; d < dim; d++) com[d] = o.center[dim * id + d];
    }
    cm.x = com[0]; cm.y = com[1]; cm.z = com[2]; cm.w = total;
    o.cm[id] = cm;
}

// Internal node from its two children (build.py:276-292 in build mode,
// refit.py:173-192 in refit mode).
// Reads a node record written by another thread of this kernel (L2, not L1).
__device__ __forceinline__ NodeCM load_cm_cg(const NodeCM* p)
{
    double2 u = __ldcg(reinterpret_cast<const double2*>(p));
    double2 v = __ldcg(reinterpret_cast<const double2*>(p) + 1);
    return NodeCM{u.x, u.y, v.x, v.y};
}

__device__ void internal_node(int32_t id, int32_t fc, int dim, bool refit, NodeOut o)
{
    NodeCM a = load_cm_cg(&o.cm[fc]);
    NodeCM b = load_cm_cg(&o.cm[fc + 1]);
    if (!refit) {
        double ext = 0.0;
        for (int d = 0; d < dim; d++) {
            double l0 = __ldcg(&o.lo[3 * fc + d]), l1 = __ldcg(&o.lo[3 * (fc + 1) + d]);
            double h0 = __ldcg(&o.hi[3 * fc + d]), h1 = __ldcg(&o.hi[3 * (fc + 1) + d]);
            double lo = l1 < l0 ? l1 : l0, hi = h1 > h0 ? h1 : h0;
            o.lo[3 * id + d] = lo;
            o.hi[3 * id + d] = hi;
            o.center[dim * id + d] = __dmul_rn(__dadd_rn(lo, hi), 0.5);
            double e = __dsub_rn(hi, lo);
            ext = (d == 0 || e > ext) ? e : ext;
        }
        o.half[id] = __dmul_rn(ext, 0.5);
        o.size[id] = __dmul_rn(2.0, o.half[id]);
    }
    double ma = a.w, mb = b.w;
    double ca[3] = {a.x, a.y, a.z}, cb[3] = {b.x, b.y, b.z};
    double total, w[3] = {0.0, 0.0, 0.0};
    if (!refit) {
        total = __dadd_rn(0.0, __dadd_rn(__dadd_rn(-0.0, ma), mb));
        for (int d = 0; d < dim; d++)
            w[d] = __dadd_rn(__dadd_rn(w[d], __dmul_rn(ma, ca[d])), __dmul_rn(mb, cb[d]));
    } else {
        total = 0.0;
        if (ma > 0) {
            total = __dadd_rn(total, ma);
            for (int d = 0; d < dim; d++) w[d] = __dadd_rn(w[d], __dmul_rn(ma, ca[d]));
        }
        if (mb > 0) {
            total = __dadd_rn(total, mb);
            for (int d = 0; d < dim; d++) w[d] = __dadd_rn(w[d], __dmul_rn(mb, cb[d]));
        }
    }
    double com[3] = {0.0, 0.0, 0.0};
    if (total > 0) {
        for (int d = 0; d < dim; d++) com[d] = __ddiv_rn(w[d], total);
    } else {
        for (int d = 0; d < dim; d++) com[d] = o.center[dim * id + d];
    }
    o.cm[id] = NodeCM{com[0], com[1], com[2], total};
}

__global__ void k_bottom_up(TreeDev t, const int32_t* __restrict__ leaf_list, int64_t num_leaves,
                            const int32_t* __restrict__ first_child,
                            const int32_t* __restrict__ start, const int32_t* __restrict__ count,
                            const int32_t* __restrict__ parent, unsigned* __restrict__ arrive,
                            NodeOut o, bool refit, const double* __restrict__ opos,
                            const double* __restrict__ omass, unsigned* __restrict__ err)
{
    for (int64_t li = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; li < num_leaves;
         li += (int64_t)gridDim.x * blockDim.x) {
        int32_t id = leaf_list[li];
        if (id < 0 || id >= t.m || start[id] < 0 || count[id] < 1 ||
            (int64_t)start[id] + count[id] > t.n) {
            atomicOr(err, kErrBadNode);
            continue;
        }
        leaf_node(id, t.dim, refit, t, opos, omass, start, count, o);
        // climb: each step is taken by the second child to arrive; a tree
        // deeper than kMaxClimb (or parent links with a cycle, possible in
        // an imported TreeData) stops with an error instead of looping
        int32_t node = id;
        for (int step = 0;; step++) {
            if (step >= kMaxClimb) { atomicOr(err, kErrBadNode); break; }
            int32_t p = parent[node];
            if (p < 0) break;
            if (p >= t.m || first_child[p] < 1 || first_child[p] + 1 >= t.m) {
                atomicOr(err, kErrBadNode);
                break;
            }
            __threadfence();
            unsigned prev = atomicAdd(&arrive[p], 1u);
            if (prev == 0) break;
            __threadfence();
            internal_node(p, first_child[p], t.dim, refit, o);
            node = p;
        }
    }
}

// Traceless quadrupole of every node about its centre of mass,
// Q_ij = sum_k m_k (3 d_i d_j - |d|^2 delta_ij), d = x_k - com (used by the
// FP32 forms with multipole "quad").  Leaves sum their particles; a parent
// adds its children's moments shifted to its own centre of mass (parallel
// axis: Q_c + M_c (3 d d^T - |d|^2 I), d = com_c - com_p).  Stored as
// (xx, yy, zz, xy, xz, yz).  Same arrival-counter climb as k_bottom_up.
__device__ __forceinline__ void quad_add(double* q, double m, double dx, double dy, double dz)
{
    const double d2 = dx * dx + dy * dy + dz * dz;
    q[0] += m * (3.0 * dx * dx - d2);
    q[1] += m * (3.0 * dy * dy - d2);
    q[2] += m * (3.0 * dz * dz - d2);
    q[3] += m * (3.0 * dx * dy);
    q[4] += m * (3.0 * dx * dz);
    q[5] += m * (3.0 * dy * dz);
}

__global__ void k_quadrupoles(TreeDev t, const int32_t* __restrict__ leaf_list, int64_t num_leaves,
                              const int32_t* __restrict__ first_child,
                              const int32_t* __restrict__ start, const int32_t* __restrict__ count,
                              const int32_t* __restrict__ parent, unsigned* __restrict__ arrive,
                              double* __restrict__ quad, unsigned* __restrict__ err)
{
    for (int64_t li = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; li < num_leaves;
         li += (int64_t)gridDim.x * blockDim.x) {
        const int32_t id = leaf_list[li];
        if (id < 0 || id >= t.m) { atomicOr(err, kErrBadNode); continue; }
        const NodeCM c = t.cm[id];
        double q[6] = {0, 0, 0, 0, 0, 0};
        const int64_t s = start[id], n = count[id];
        for (int64_t i = s; i < s + n; i++)
            quad_add(q, t.sm[i], t.sx[i] - c.x, t.sy[i] - c.y, t.dim == 3 ? t.sz[i] - c.z : 0.0);
        for (int k = 0; k < 6; k++) quad[6 * (int64_t)id + k] = q[k];
        int32_t node = id;
        for (int step = 0;; step++) {
            if (step >= kMaxClimb) { atomicOr(err, kErrBadNode); break; }
            const int32_t p = parent[node];
            if (p < 0) break;
            if (p >= t.m || first_child[p] < 1 || first_child[p] + 1 >= t.m) {
                atomicOr(err, kErrBadNode);
                break;
            }
            __threadfence();
            if (atomicAdd(&arrive[p], 1u) == 0) break;
            __threadfence();
            const NodeCM cp = t.cm[p];
            double qp[6] = {0, 0, 0, 0, 0, 0};
            for (int j = 0; j < 2; j++) {
                const int32_t ch = first_child[p] + j;
                const double2 a = __ldcg(reinterpret_cast<const double2*>(&t.cm[ch]));
                const double2 b = __ldcg(reinterpret_cast<const double2*>(&t.cm[ch]) + 1);
                for (int k = 0; k < 6; k++) qp[k] += __ldcg(&quad[6 * (int64_t)ch + k]);
                quad_add(qp, b.y, a.x - cp.x, a.y - cp.y, t.dim == 3 ? b.x - cp.z : 0.0);
            }
            for (int k = 0; k < 6; k++) quad[6 * (int64_t)p + k] = qp[k];
            node = p;
        }
    }
}

int launch_quadrupoles(const TreeDev& t, const int32_t* leaf_list, int64_t num_leaves,
                       const int32_t* first_child, const int32_t* start, const int32_t* count,
                       const int32_t* parent, unsigned* arrive, double* quad, unsigned* err,
                       cudaStream_t s)
{
    BHUT_CUDA(cudaMemsetAsync(arrive, 0, sizeof(unsigned) * (size_t)t.m, s));
    k_quadrupoles<<<grid_for(num_leaves, 128), 128, 0, s>>>(t, leaf_list, num_leaves, first_child,
                                                            start, count, parent, arrive, quad,
                                                            err);
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    return kOk;
}

// Refit-vs-rebuild test of refit.py:236-249: any particle with
// max_axis |x - root_center| > 1.1 * root_half_size forces a rebuild.
__global__ void k_outside_root(const double* __restrict__ pos, int64_t n, int dim,
                               const double* __restrict__ center0, const double* __restrict__ half0,
                               unsigned* __restrict__ flag)
{
    double lim = __dmul_rn(1.1, *half0);
    bool out = false;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        double mx = fabs(__dsub_rn(pos[i * dim], center0[0]));
        for (int d = 1; d < dim; d++) {
            double v = fabs(__dsub_rn(pos[i * dim + d], center0[d]));
            mx = v > mx ? v : mx;
        }
        out |= (mx > lim) || !(mx == mx);
    }
    if (__any_sync(0xffffffffu, out) && (threadIdx.x & 31) == 0) atomicOr(flag, 1u);
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
int make_topo_tables(int64_t n, int leaf_size, TopoTables* t)
{
    if (n <= 0 || leaf_size <= 0) { set_error("invalid topology request"); return kInvalid; }
    t->n = n;
    t->leaf_size = leaf_size;
    int depth = 0;
    while (true) {
        int64_t mx = (n + (1ll << depth) - 1) >> depth;   // ceil(n / 2^depth)
        if (mx <= leaf_size) break;
        depth++;
        if (depth >= kMaxDepth - 1) { set_error("tree too deep"); return kInvalid; }
    }
    t->depth = depth;
    for (int d = 0; d <= depth + 1 && d < kMaxDepth; d++) t->cnt_lo[d] = n >> d;
    // internal-node counts bottom-up: I(c) = 0 if c <= L else 1 + I(c/2) + I(c - c/2)
    for (int d = depth + 1; d >= 0; d--) {
        if (d >= kMaxDepth) continue;
        for (int v = 0; v < 2; v++) {
            int64_t c = t->cnt_lo[d] + v;
            if (c <= leaf_size) { t->internal[d][v] = 0; continue; }
            int64_t h = c / 2, r = c - h;
            int64_t lo = t->cnt_lo[d + 1];
            t->internal[d][v] = 1 + t->internal[d + 1][h - lo] + t->internal[d + 1][r - lo];
        }
    }
    int64_t ni = t->internal[0][0];
    t->num_nodes = 1 + 2 * ni;
    t->num_leaves = t->num_nodes - ni;
    t->slots = (2ll << depth) - 1;
    return kOk;
}

int launch_bbox(const double* pos, const double* mass, int64_t n, int dim, double* partial,
                unsigned* counter, double* box, unsigned* err, cudaStream_t s)
{
    unsigned g = grid_for(n, kBoxThreads, kBoxMaxBlocks);
    k_bbox<<<g, kBoxThreads, 0, s>>>(pos, mass, n, dim, partial, counter, box, err);
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    return kOk;
}

int launch_morton(const double* pos, int64_t n, int dim, const double* box, uint64_t* keys,
                  int32_t* idx, cudaStream_t s)
{
    k_morton<<<grid_for(n, 256), 256, 0, s>>>(pos, n, dim, box, keys, idx);
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    return kOk;
}

int launch_gather(const double* pos, const double* mass, const int32_t* perm, int64_t n, int dim,
                  double* sx, double* sy, double* sz, double* sm, cudaStream_t s)
{
    k_gather_sorted<<<grid_for(n, 256), 256, 0, s>>>(pos, mass, perm, n, dim, sx, sy, sz, sm);
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    return kOk;
}

int launch_topology(const TopoTables& tt, int32_t* first_child, int32_t* start, int32_t* count,
                    int32_t* parent, int32_t* leaf_list, unsigned* leaf_counter, unsigned* err,
                    cudaStream_t s)
{
    BHUT_CUDA(cudaMemsetAsync(leaf_counter, 0, sizeof(unsigned), s));
    k_topology<<<grid_for(tt.slots, 256), 256, 0, s>>>(tt, first_child, start, count, parent,
                                                       leaf_list, leaf_counter, err);
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    return kOk;
}

int launch_bottom_up(const TreeDev& t, const int32_t* leaf_list, int64_t num_leaves,
                     const int32_t* first_child, const int32_t* start, const int32_t* count,
                     const int32_t* parent, unsigned* arrive, NodeOut o, bool refit,
                     const double* opos, const double* omass, unsigned* err, cudaStream_t s)
{
    BHUT_CUDA(cudaMemsetAsync(arrive, 0, sizeof(unsigned) * (size_t)t.m, s));
    k_bottom_up<<<grid_for(num_leaves, 128), 128, 0, s>>>(t, leaf_list, num_leaves, first_child,
                                                          start, count, parent, arrive, o, refit,
                                                          opos, omass, err);
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    return kOk;
}

int launch_outside_root(const double* pos, int64_t n, int dim, const double* center0,
                        const double* half0, unsigned* flag, cudaStream_t s)
{
    k_outside_root<<<grid_for(n, 256, 152u * 4u), 256, 0, s>>>(pos, n, dim, center0, half0, flag);
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    return kOk;
}

}  // namespace bhut
