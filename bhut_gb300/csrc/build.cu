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
// K1: bounding box.  The position array is read as a flat array of n * dim
// doubles; the grid stride is a multiple of 6, so each thread sees one axis.
// Minima and maxima are taken on order-preserving integer images of the
// doubles (the FP64 pipe runs at 1/64 of the integer pipes here), which
// give the same values as FP64 comparisons (-0.0 and +0.0 aside, which
// compare equal).  Optionally the kernel also copies positions and masses
// to staging buffers (one read for the copy, the finiteness check and the
// box).  Block partials; the last block to finish reduces them (no block
// waits on another) and adds the extents' reciprocals for the Morton
// quantiser and per-axis NaN flags.
// ---------------------------------------------------------------------------
constexpr int kBoxThreads = 192;   // a multiple of 6 and of 32


__global__ void __launch_bounds__(kBoxThreads)
k_bbox(const double* __restrict__ pos, const double* __restrict__ mass, int64_t n, int dim,
       double* __restrict__ pos_copy, double* __restrict__ mass_copy,
       double* __restrict__ partial, unsigned* __restrict__ done_counter, double* __restrict__ box,
       unsigned* __restrict__ err)
{
    const int tid = threadIdx.x;
    const int64_t first = blockIdx.x * (int64_t)kBoxThreads + tid;
    const int64_t stride = (int64_t)gridDim.x * kBoxThreads;   // multiple of 6
    const int64_t total = n * dim;
    const int axis = (int)(first % dim);
    const uint64_t* __restrict__ p = reinterpret_cast<const uint64_t*>(pos);
    uint64_t* __restrict__ pc = reinterpret_cast<uint64_t*>(pos_copy);
    uint64_t lo = ~0ull, hi = 0ull;
    bool bad = false, nan = false;
    // batches of kBoxBatch loads are issued before any store of the copy
    // (the copy does not alias the input, but the compiler cannot know)
    constexpr int kBoxBatch = 8;
    for (int64_t j0 = first; j0 < total; j0 += kBoxBatch * stride) {
        uint64_t b[kBoxBatch];
#pragma unroll
        for (int u = 0; u < kBoxBatch; u++) {
            const int64_t j = j0 + u * stride;
            b[u] = j < total ? __ldg(p + j) : 0ull;
        }
#pragma unroll
        for (int u = 0; u < kBoxBatch; u++) {
            const int64_t j = j0 + u * stride;
            if (j < total) {
                if (pc) pc[j] = b[u];
                bad |= !finite_bits(b[u]);
                nan |= (b[u] & 0x7FFFFFFFFFFFFFFFull) > 0x7FF0000000000000ull;
                const uint64_t k = ord_key(b[u]);
                lo = k < lo ? k : lo;
                hi = k > hi ? k : hi;
            }
        }
    }
    uint64_t mm = 0ull;   // |mass| bits: non-negative doubles order as integers
    bool mdiff = false;   // a mass differs from mass[0] (bit for bit)
    if (mass) {
        const uint64_t* __restrict__ q = reinterpret_cast<const uint64_t*>(mass);
        const uint64_t m0b = __ldg(q);
        uint64_t* __restrict__ qc = reinterpret_cast<uint64_t*>(mass_copy);
        for (int64_t i0 = first; i0 < n; i0 += kBoxBatch * stride) {
            uint64_t b[kBoxBatch];
#pragma unroll
            for (int u = 0; u < kBoxBatch; u++) {
                const int64_t i = i0 + u * stride;
                b[u] = i < n ? __ldg(q + i) : 0ull;
            }
#pragma unroll
            for (int u = 0; u < kBoxBatch; u++) {
                const int64_t i = i0 + u * stride;
                if (i < n) {
                    if (qc) qc[i] = b[u];
                    bad |= !finite_bits(b[u]);
                    const uint64_t a = b[u] & 0x7FFFFFFFFFFFFFFFull;
                    mm = a > mm ? a : mm;
                    mdiff |= b[u] != m0b;
                }
            }
        }
    }
    if (__any_sync(0xffffffffu, bad) && (tid & 31) == 0) atomicOr(err, kErrNonFinite);
    __shared__ uint64_t s_lo[kBoxThreads], s_hi[kBoxThreads], s_m[kBoxThreads];
    __shared__ bool s_last;
    __shared__ unsigned s_nan;   // bit d: axis d holds a NaN
    if (tid == 0) s_nan = 0;
    s_lo[tid] = lo;
    s_hi[tid] = hi;
    s_m[tid] = mm;
    __syncthreads();
    if (nan) atomicOr(&s_nan, 1u << axis);
    if (mdiff) atomicOr(&s_nan, 8u);   // bit 3: masses not all equal
    // thread d < dim reduces its axis (the threads with tid = d (mod dim):
    // the block's first index is a multiple of 6); thread 3 the masses
    if (tid < dim) {
        uint64_t l = ~0ull, h = 0ull;
        for (int t = tid; t < kBoxThreads; t += dim) {
            l = s_lo[t] < l ? s_lo[t] : l;
            h = s_hi[t] > h ? s_hi[t] : h;
        }
        partial[blockIdx.x * 8 + tid] = __longlong_as_double((long long)l);
        partial[blockIdx.x * 8 + 3 + tid] = __longlong_as_double((long long)h);
    } else if (tid == 3) {
        uint64_t m = 0ull;
        for (int t = 0; t < kBoxThreads; t++) m = s_m[t] > m ? s_m[t] : m;
        partial[blockIdx.x * 8 + 6] = __longlong_as_double((long long)m);
    }
    __syncthreads();
    if (tid == 0) {
        partial[blockIdx.x * 8 + 7] = (double)s_nan;
        __threadfence();
        const unsigned ticket = atomicAdd(done_counter, 1u);
        s_last = (ticket == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return;
    // last block: reduce the partials (ordered images; |mass| bits), all
    // threads striding over the blocks, then across the block
    __threadfence();
    uint64_t a[7];
    for (int k = 0; k < 3; k++) { a[k] = ~0ull; a[3 + k] = 0ull; }
    a[6] = 0ull;
    unsigned nanmask = 0;
    for (unsigned g = tid; g < gridDim.x; g += kBoxThreads) {
        for (int k = 0; k < 7; k++) {
            const uint64_t v = (uint64_t)__double_as_longlong(__ldcg(&partial[g * 8 + k]));
            if (k < 3) a[k] = v < a[k] ? v : a[k];
            else a[k] = v > a[k] ? v : a[k];
        }
        nanmask |= (unsigned)__ldcg(&partial[g * 8 + 7]);
    }
    constexpr int kBoxWarps = kBoxThreads / 32;
    __shared__ uint64_t s_red[7][kBoxWarps];
    for (int k = 0; k < 7; k++) {
        for (int o = 16; o > 0; o >>= 1) {
            const uint64_t v = __shfl_down_sync(0xffffffffu, a[k], o);
            if (k < 3) a[k] = v < a[k] ? v : a[k];
            else a[k] = v > a[k] ? v : a[k];
        }
        if ((tid & 31) == 0) s_red[k][tid >> 5] = a[k];
    }
    if (nanmask) atomicOr(&s_nan, nanmask << 4);   // bits 4..6: the grid's NaN axes, 7: masses differ
    __syncthreads();
    if (tid < 7) {
        uint64_t acc = s_red[tid][0];
        for (int w = 1; w < kBoxWarps; w++) {
            const uint64_t v = s_red[tid][w];
            if (tid < 3) acc = v < acc ? v : acc;
            else acc = v > acc ? v : acc;
        }
        const int d = tid < 3 ? tid : tid - 3;
        if (tid == 6)
            box[6] = __longlong_as_double((long long)acc);
        else if (d < dim)
            box[tid] = __longlong_as_double((long long)ord_inv(acc));
        else
            box[tid] = tid < 3 ? INFINITY : -INFINITY;
    }
    __syncthreads();
    // per axis the reciprocal of the extent that the Morton quantiser uses
    // (box[8 + d]), whether an axis has zero extent (box[11]) and which axes
    // hold a NaN (box[12 + d])
    if (tid == 0) {
        bool degenerate = false;
        for (int d = 0; d < 3; d++) {
            double r = 1.0;
            if (d < dim) {
                const double e = __dsub_rn(box[3 + d], box[d]);
                degenerate |= !(e > 0.0);
                r = e > 0.0 ? __drcp_rn(e) : 1.0;
            }
            box[8 + d] = r;
        }
        box[11] = degenerate ? 1.0 : 0.0;
        for (int d = 0; d < 3; d++) box[12 + d] = (s_nan >> (4 + d)) & 1u ? 1.0 : 0.0;
        // box[15]: every particle has the same positive, finite mass (the
        // float-float traversal then measures masses in units of it)
        bool unit = false;
        if (mass && !((s_nan >> 7) & 1u)) {
            const double m0 = mass[0];
            unit = m0 > 0.0 && finite_bits((uint64_t)__double_as_longlong(m0));
        }
        box[15] = unit ? 1.0 : 0.0;
        *done_counter = 0;
    }
}

// ---------------------------------------------------------------------------
// K2: Morton keys (input order) and the identity payload for the sort.
// ---------------------------------------------------------------------------
template <int dim>
__global__ void k_morton(const double* __restrict__ pos, int64_t n,
                         const double* __restrict__ box, uint64_t* __restrict__ keys,
                         int32_t* __restrict__ idx)
{
    double pmin[3], ext[3], off[3], rcp[3];
    for (int d = 0; d < dim; d++) {
        pmin[d] = box[d];
        double e = __dsub_rn(box[3 + d], box[d]);
        ext[d] = e <= 0 ? 1.0 : e;
        off[d] = e <= 0 ? 0.5 : 0.0;
        rcp[d] = box[8 + d];   // RN(1 / extent), from the bounding-box kernel
    }
    const bool degenerate = box[11] != 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t key;
        if (degenerate) {   // an axis of zero extent (uniform branch)
            if (dim == 3) {
                key = morton3(quantise(pos[3 * i], pmin[0], ext[0], off[0]),
                              quantise(pos[3 * i + 1], pmin[1], ext[1], off[1]),
                              quantise(pos[3 * i + 2], pmin[2], ext[2], off[2]));
            } else {
                key = morton2(quantise(pos[2 * i], pmin[0], ext[0], off[0]),
                              quantise(pos[2 * i + 1], pmin[1], ext[1], off[1]));
            }
        } else if (dim == 3) {
            key = morton3(quantise_rcp(pos[3 * i], pmin[0], ext[0], rcp[0]),
                          quantise_rcp(pos[3 * i + 1], pmin[1], ext[1], rcp[1]),
                          quantise_rcp(pos[3 * i + 2], pmin[2], ext[2], rcp[2]));
        } else {
            key = morton2(quantise_rcp(pos[2 * i], pmin[0], ext[0], rcp[0]),
                          quantise_rcp(pos[2 * i + 1], pmin[1], ext[1], rcp[1]));
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
// DIM is a template parameter so that the per-axis accumulators stay in
// registers (a runtime axis index would place them in local memory).
template <int DIM>
__device__ void leaf_node(int32_t id, bool refit, const TreeDev& t,
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
        // AABB on order-preserving integer images (same values as FP64
        // comparisons; the FP64 pipe is the scarce one); loads run ahead of
        // the row-order sums
        uint64_t klo[3] = {~0ull, ~0ull, ~0ull}, khi[3] = {0ull, 0ull, 0ull};
        const double* axes[3] = {t.sx, t.sy, t.sz};
#pragma unroll 4
        for (int64_t i = 0; i < c; i++) {
            const double mi = t.sm[s + i];
            for (int d = 0; d < DIM; d++) {
                const double v = axes[d][s + i];
                const uint64_t k = ord_key((uint64_t)__double_as_longlong(v));
                klo[d] = k < klo[d] ? k : klo[d];
                khi[d] = k > khi[d] ? k : khi[d];
                acc[d] = __dadd_rn(acc[d], __dmul_rn(mi, v));
            }
        }
        double lo[3], hi[3];
        for (int d = 0; d < DIM; d++) {
            lo[d] = __longlong_as_double((long long)ord_inv(klo[d]));
            hi[d] = __longlong_as_double((long long)ord_inv(khi[d]));
        }
        double ext = 0.0;
        for (int d = 0; d < DIM; d++) {
            o.lo[3 * id + d] = lo[d];
            o.hi[3 * id + d] = hi[d];
            o.center[DIM * id + d] = __dmul_rn(__dadd_rn(lo[d], hi[d]), 0.5);
            double e = __dsub_rn(hi[d], lo[d]);
            ext = (d == 0 || e > ext) ? e : ext;
        }
        o.half[id] = __dmul_rn(ext, 0.5);
        o.size[id] = __dmul_rn(2.0, o.half[id]);
    } else {
        auto ld = [&](int64_t i) { return omass[t.perm[s + i]]; };
        total = __dadd_rn(0.0, pairwise_sum(ld, c));
#pragma unroll 4
        for (int64_t i = 0; i < c; i++) {
            int64_t p = t.perm[s + i];
            double mi = omass[p];
            for (int d = 0; d < DIM; d++)
                acc[d] = __dadd_rn(acc[d], __dmul_rn(mi, opos[p * DIM + d]));
        }
    }
    NodeCM cm;
    double com[3];
    for (int d = 0; d < 3; d++) com[d] = 0.0;
    if (total > 0) {
        for (int d = 0; d < DIM; d++) com[d] = __ddiv_rn(acc[d], total);
    } else {
        for (int d = 0; d < DIM; d++) com[d] = o.center[DIM * id + d];
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

template <int DIM>
__device__ void internal_node(int32_t id, int32_t fc, bool refit, NodeOut o)
{
    NodeCM a = load_cm_cg(&o.cm[fc]);
    NodeCM b = load_cm_cg(&o.cm[fc + 1]);
    if (!refit) {
        double ext = 0.0;
        for (int d = 0; d < DIM; d++) {
            const uint64_t l0 = ord_key((uint64_t)__double_as_longlong(__ldcg(&o.lo[3 * fc + d])));
            const uint64_t l1 = ord_key((uint64_t)__double_as_longlong(__ldcg(&o.lo[3 * (fc + 1) + d])));
            const uint64_t h0 = ord_key((uint64_t)__double_as_longlong(__ldcg(&o.hi[3 * fc + d])));
            const uint64_t h1 = ord_key((uint64_t)__double_as_longlong(__ldcg(&o.hi[3 * (fc + 1) + d])));
            const double lo = __longlong_as_double((long long)ord_inv(l1 < l0 ? l1 : l0));
            const double hi = __longlong_as_double((long long)ord_inv(h1 > h0 ? h1 : h0));
            o.lo[3 * id + d] = lo;
            o.hi[3 * id + d] = hi;
            o.center[DIM * id + d] = __dmul_rn(__dadd_rn(lo, hi), 0.5);
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
        for (int d = 0; d < DIM; d++)
            w[d] = __dadd_rn(__dadd_rn(w[d], __dmul_rn(ma, ca[d])), __dmul_rn(mb, cb[d]));
    } else {
        total = 0.0;
        if (ma > 0) {
            total = __dadd_rn(total, ma);
            for (int d = 0; d < DIM; d++) w[d] = __dadd_rn(w[d], __dmul_rn(ma, ca[d]));
        }
        if (mb > 0) {
            total = __dadd_rn(total, mb);
            for (int d = 0; d < DIM; d++) w[d] = __dadd_rn(w[d], __dmul_rn(mb, cb[d]));
        }
    }
    double com[3] = {0.0, 0.0, 0.0};
    if (total > 0) {
        for (int d = 0; d < DIM; d++) com[d] = __ddiv_rn(w[d], total);
    } else {
        for (int d = 0; d < DIM; d++) com[d] = o.center[DIM * id + d];
    }
    o.cm[id] = NodeCM{com[0], com[1], com[2], total};
}

// Leaves are taken in groups of kBuThreads consecutive entries of the leaf
// list (one thread each).  Inside the group the lowest kBuLevels levels are
// merged in shared memory: at level j slot k holds the node covering leaves
// [k 2^j, (k+1) 2^j) of the group; thread t < slots / 2 pairs slots 2t and
// 2t + 1 and, when they are the two children of one node, computes that node
// into slot t (compacted, so the FP64 work of a level runs on as few warps
// as possible; block barriers order the children's writes; no atomics, no
// device-wide fences).  A node whose sibling is not in its pair -- it lies
// in another group, or the tree is irregular there -- goes to the frontier
// list, from which k_bottom_up_top finishes the tree.
#ifndef BHUT_BU_LEVELS
#define BHUT_BU_LEVELS 8   // tuning: leaves per group = 2^levels
#endif
constexpr int kBuLevels = BHUT_BU_LEVELS;
constexpr int kBuThreads = 1 << kBuLevels;

__device__ __forceinline__ bool bad_parent(const TreeDev& t, const int32_t* first_child, int32_t p)
{
    return p >= t.m || (p >= 0 && (first_child[p] < 1 || first_child[p] + 1 >= t.m));
}

__device__ __forceinline__ void hand_over(int32_t node, int32_t* frontier, unsigned* frontier_count,
                                          int64_t cap, unsigned* err)
{
    const unsigned k = atomicAdd(frontier_count, 1u);
    if (k < (unsigned)cap) frontier[k] = node;
    else atomicOr(err, kErrBadNode);
}

// Node operations of a bottom-up pass: the moments (build and refit modes)
// or the quadrupoles.
template <int DIM>
struct MomentOps {
    TreeDev t;
    NodeOut o;
    bool refit;
    const double* opos;
    const double* omass;
    const int32_t* start;
    const int32_t* count;
    __device__ void leaf(int32_t id) const { leaf_node<DIM>(id, refit, t, opos, omass, start, count, o); }
    __device__ void internal(int32_t p, int32_t fc) const { internal_node<DIM>(p, fc, refit, o); }
};

template <class Ops>
__global__ void __launch_bounds__(kBuThreads)
k_bottom_up(Ops ops, TreeDev t, const int32_t* __restrict__ leaf_list, int64_t num_leaves,
            const int32_t* __restrict__ first_child, const int32_t* __restrict__ start,
            const int32_t* __restrict__ count, const int32_t* __restrict__ parent,
            int32_t* __restrict__ frontier, unsigned* __restrict__ frontier_count,
            unsigned* __restrict__ err)
{
    __shared__ int32_t s_node[kBuThreads];
    const int tid = threadIdx.x;
    for (int64_t base = (int64_t)blockIdx.x * kBuThreads; base < num_leaves;
         base += (int64_t)gridDim.x * kBuThreads) {
        const int64_t li = base + tid;
        const int32_t id = li < num_leaves ? leaf_list[li] : -1;
        bool alive = li < num_leaves;
        if (alive && (id < 0 || id >= t.m || start[id] < 0 || count[id] < 1 ||
                      (int64_t)start[id] + count[id] > t.n)) {
            atomicOr(err, kErrBadNode);
            alive = false;
        }
        if (alive) ops.leaf(id);
        s_node[tid] = alive ? id : -1;
        __syncthreads();
        for (int j = 0, slots = kBuThreads; j < kBuLevels; j++, slots >>= 1) {
            int32_t out = -1;
            if (tid < slots / 2) {
                const int32_t a = s_node[2 * tid], b = s_node[2 * tid + 1];
                int32_t pa = -1, pb = -1;
                if (a >= 0) {
                    pa = parent[a];
                    if (bad_parent(t, first_child, pa)) { atomicOr(err, kErrBadNode); pa = -2; }
                }
                if (b >= 0) {
                    pb = parent[b];
                    if (bad_parent(t, first_child, pb)) { atomicOr(err, kErrBadNode); pb = -2; }
                }
                if (pa >= 0 && pa == pb) {
                    ops.internal(pa, first_child[pa]);
                    out = pa;
                } else {   // parents completed elsewhere (or roots: nothing to do)
                    if (pa >= 0) hand_over(a, frontier, frontier_count, num_leaves, err);
                    if (pb >= 0) hand_over(b, frontier, frontier_count, num_leaves, err);
                }
            }
            __syncthreads();
            if (tid < slots / 2) s_node[tid] = out;
            __syncthreads();
        }
        if (tid == 0 && s_node[0] >= 0) {
            const int32_t p = parent[s_node[0]];
            if (bad_parent(t, first_child, p)) atomicOr(err, kErrBadNode);
            else if (p >= 0) hand_over(s_node[0], frontier, frontier_count, num_leaves, err);
        }
        __syncthreads();
    }
}

// The rest of the tree, from the frontier nodes up, by one block: each
// climb step is taken by the second child to arrive at a parent (arrival
// counters).  All climbers run in this block, so block-scope fences order
// a child's writes before its arrival, and while the frontier is small the
// counters live in a shared-memory hash table keyed by node id (a frontier
// of f nodes has f - 1 ancestors to count at most); a larger frontier
// counts in global memory.  A climb longer than kMaxClimb (parent links
// with a cycle, possible in an imported TreeData) stops with an error
// instead of looping.
constexpr int kBuTopThreads = 1024;
constexpr int kBuTopHash = 4096;   // shared counters: frontiers of up to 2048 nodes

template <class Ops>
__global__ void __launch_bounds__(kBuTopThreads)
k_bottom_up_top(Ops ops, TreeDev t, const int32_t* __restrict__ first_child,
                const int32_t* __restrict__ parent, unsigned* __restrict__ arrive,
                const int32_t* __restrict__ frontier,
                const unsigned* __restrict__ frontier_count, int64_t cap,
                unsigned* __restrict__ err)
{
    __shared__ int32_t s_key[kBuTopHash];
    __shared__ unsigned s_cnt[kBuTopHash];
    const unsigned nf = min(*frontier_count, (unsigned)cap);
    const bool shared_counters = nf <= kBuTopHash / 2;
    for (int i = threadIdx.x; i < kBuTopHash; i += blockDim.x) {
        s_key[i] = -1;
        s_cnt[i] = 0;
    }
    __syncthreads();
    for (unsigned f = threadIdx.x; f < nf; f += blockDim.x) {
        int32_t node = frontier[f];
        for (int step = 0;; step++) {
            if (step >= kMaxClimb || node < 0 || node >= t.m) { atomicOr(err, kErrBadNode); break; }
            const int32_t p = parent[node];
            if (p < 0) break;
            if (bad_parent(t, first_child, p)) { atomicOr(err, kErrBadNode); break; }
            __threadfence_block();
            unsigned prev;
            if (shared_counters) {
                // linear probing from a multiplicative hash; at most f - 1
                // keys in 2f slots, so a free or matching slot is found
                unsigned h = ((unsigned)p * 2654435761u) >> 20;   // 12 bits
                int probes = 0;
                for (;; h = (h + 1) & (kBuTopHash - 1)) {
                    const int32_t k = atomicCAS(&s_key[h], -1, p);
                    if (k == -1 || k == p) break;
                    if (++probes >= kBuTopHash) break;
                }
                if (probes >= kBuTopHash) { atomicOr(err, kErrBadNode); break; }
                prev = atomicAdd(&s_cnt[h], 1u);
            } else {
                prev = atomicAdd_block(&arrive[p], 1u);
            }
            if (prev == 0) break;
            __threadfence_block();
            ops.internal(p, first_child[p]);
            node = p;
        }
    }
}

template <class Ops>
int launch_climb(const Ops& ops, const TreeDev& t, const int32_t* leaf_list, int64_t num_leaves,
                 const int32_t* first_child, const int32_t* start, const int32_t* count,
                 const int32_t* parent, unsigned* arrive, int32_t* frontier,
                 unsigned* frontier_count, unsigned* err, cudaStream_t s)
{
    BHUT_CUDA(cudaMemsetAsync(arrive, 0, sizeof(unsigned) * (size_t)t.m, s));
    BHUT_CUDA(cudaMemsetAsync(frontier_count, 0, sizeof(unsigned), s));
    const unsigned groups = (unsigned)((num_leaves + kBuThreads - 1) / kBuThreads);
    k_bottom_up<Ops><<<groups < 152u * 8u ? groups : 152u * 8u, kBuThreads, 0, s>>>(
        ops, t, leaf_list, num_leaves, first_child, start, count, parent, frontier,
        frontier_count, err);
    k_bottom_up_top<Ops><<<1, kBuTopThreads, 0, s>>>(ops, t, first_child, parent, arrive,
                                                     frontier, frontier_count, num_leaves, err);
    BHUT_CUDA(cudaGetLastError());
    note_launches(2);
    return kOk;
}

// Sort keys for ordering the leaf list by first particle (once per topology).
__global__ void k_leaf_keys(const int32_t* __restrict__ leaf_list, int64_t num_leaves,
                            const int32_t* __restrict__ start, uint64_t* __restrict__ keys)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < num_leaves;
         i += (int64_t)gridDim.x * blockDim.x)
        keys[i] = (uint64_t)(uint32_t)start[leaf_list[i]];
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

struct QuadOps {
    TreeDev t;
    double* quad;
    const int32_t* start;
    const int32_t* count;
    __device__ void leaf(int32_t id) const
    {
        const NodeCM c = t.cm[id];
        double q[6] = {0, 0, 0, 0, 0, 0};
        const int64_t s = start[id], n = count[id];
        for (int64_t i = s; i < s + n; i++)
            quad_add(q, t.sm[i], t.sx[i] - c.x, t.sy[i] - c.y, t.dim == 3 ? t.sz[i] - c.z : 0.0);
        for (int k = 0; k < 6; k++) quad[6 * (int64_t)id + k] = q[k];
    }
    __device__ void internal(int32_t p, int32_t fc) const
    {
        const NodeCM cp = t.cm[p];
        double qp[6] = {0, 0, 0, 0, 0, 0};
        for (int j = 0; j < 2; j++) {
            const int32_t ch = fc + j;
            const double2 a = __ldcg(reinterpret_cast<const double2*>(&t.cm[ch]));
            const double2 b = __ldcg(reinterpret_cast<const double2*>(&t.cm[ch]) + 1);
            for (int k = 0; k < 6; k++) qp[k] += __ldcg(&quad[6 * (int64_t)ch + k]);
            quad_add(qp, b.y, a.x - cp.x, a.y - cp.y, t.dim == 3 ? b.x - cp.z : 0.0);
        }
        for (int k = 0; k < 6; k++) quad[6 * (int64_t)p + k] = qp[k];
    }
};

int launch_quadrupoles(const TreeDev& t, const int32_t* leaf_list, int64_t num_leaves,
                       const int32_t* first_child, const int32_t* start, const int32_t* count,
                       const int32_t* parent, unsigned* arrive, double* quad, int32_t* frontier,
                       unsigned* frontier_count, unsigned* err, cudaStream_t s)
{
    return launch_climb(QuadOps{t, quad, start, count}, t, leaf_list, num_leaves, first_child,
                        start, count, parent, arrive, frontier, frontier_count, err, s);
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
    return launch_stage_bbox(pos, mass, n, dim, nullptr, nullptr, partial, counter, box, err, s);
}

int launch_stage_bbox(const double* pos, const double* mass, int64_t n, int dim, double* pos_copy,
                      double* mass_copy, double* partial, unsigned* counter, double* box,
                      unsigned* err, cudaStream_t s)
{
    unsigned g = grid_for(n * dim, kBoxThreads * 4, kBoxMaxBlocks);
    k_bbox<<<g, kBoxThreads, 0, s>>>(pos, mass, n, dim, pos_copy, mass_copy, partial, counter,
                                     box, err);
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    return kOk;
}

int launch_morton(const double* pos, int64_t n, int dim, const double* box, uint64_t* keys,
                  int32_t* idx, cudaStream_t s)
{
    if (dim == 3) k_morton<3><<<grid_for(n, 256), 256, 0, s>>>(pos, n, box, keys, idx);
    else k_morton<2><<<grid_for(n, 256), 256, 0, s>>>(pos, n, box, keys, idx);
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

int order_leaves(int32_t* leaf_list, int64_t num_leaves, const int32_t* start, uint64_t* keys,
                 void* sort_scratch, cudaStream_t s)
{
    k_leaf_keys<<<grid_for(num_leaves, 256), 256, 0, s>>>(leaf_list, num_leaves, start, keys);
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    return radix_sort_pairs(keys, leaf_list, num_leaves, 31, sort_scratch, s);
}

int launch_bottom_up(const TreeDev& t, const int32_t* leaf_list, int64_t num_leaves,
                     const int32_t* first_child, const int32_t* start, const int32_t* count,
                     const int32_t* parent, unsigned* arrive, NodeOut o, bool refit,
                     const double* opos, const double* omass, int32_t* frontier,
                     unsigned* frontier_count, unsigned* err, cudaStream_t s)
{
    if (t.dim == 3)
        return launch_climb(MomentOps<3>{t, o, refit, opos, omass, start, count}, t, leaf_list,
                            num_leaves, first_child, start, count, parent, arrive, frontier,
                            frontier_count, err, s);
    return launch_climb(MomentOps<2>{t, o, refit, opos, omass, start, count}, t, leaf_list,
                        num_leaves, first_child, start, count, parent, arrive, frontier,
                        frontier_count, err, s);
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
