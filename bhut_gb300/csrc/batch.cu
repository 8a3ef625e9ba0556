// Batched form: many independent N-body systems solved in one pass.
//
// The systems are concatenated (CSR offsets).  The build is segmented, and
// every per-solve kernel spreads its work over the particles (or nodes), not
// over the systems, so that one large system is not left to one block:
//   k_seg_acc_init    per-system accumulators cleared
//   k_seg_bbox_chunks one block per chunk of <= kSegChunk particles of one
//                     system: box, max |m|, equal-mass test, merged into the
//                     system's accumulators with 64-bit integer atomics
//   k_seg_box_finish  per system: box, Morton quantiser data, frame
//   k_seg_morton      per particle: Morton key in its system's box
//   radix_sort_pairs  by Morton key, then (stable) by system id
//   k_gather_sorted   sorted SoA (global)
//   k_seg_topology    one block per system: the count-split topology of
//                     bhut/tree/build.py:110-212 for that system's N, ids
//                     offset into one forest (cached while the layout holds)
//   k_bottom_up       shared with the single-tree engine (leaves of all
//                     systems climb their own tree)
//   k_seg_ff_particles, k_seg_ff_nodes
//                     per particle / node: float-float copies in the system's
//                     frame
// and the traversal is one persistent kernel: every warp pulls
// (system, target chunk) tasks from a global atomic counter (heaviest systems
// first) until the queue is empty -- no warp waits on another.  Each task is
// the warp-cooperative walk of the single-tree kernels, rooted at the
// system's root; with TPW = 16 two lanes share a target and split its pair
// loop.  All launches of a solve can be captured in one CUDA graph.
#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/bhut_gb300.h"
#include "fast.cuh"

namespace bhut {
bool is_device_pointer(const void* p);
}

using namespace bhut;

namespace {

constexpr int kSegThreads = 256;
constexpr int kBatchWarps = 4;
constexpr int kBatchThreads = kBatchWarps * kWarp;

// ---------------------------------------------------------------------------
// segmented build kernels
// ---------------------------------------------------------------------------
// Per-system accumulators (kSegAcc x uint64 per system): ordered images of
// min x, y, z and of max x, y, z, the bits of max |mass|, flags (bit 0: a
// mass differs from the system's first, bit 1: a particle lies beyond 1.1x
// the system's root box).
constexpr int kSegAcc = 8;
constexpr int kSegChunk = 4096;   // particles per block of the chunked box
// Per-system box (kSegBox doubles): min (0..2), max (3..5), max |m| (6),
// equal positive masses (7), RN(1 / extent) (8..10), zero extent on some
// axis (11), extent (12..14; 1 for a zero extent).
constexpr int kSegBox = 16;

__global__ void k_seg_acc_init(uint64_t* __restrict__ acc, int64_t ns)
{
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < ns;
         s += (int64_t)gridDim.x * blockDim.x) {
        uint64_t* a = acc + kSegAcc * s;
        a[0] = a[1] = a[2] = ~0ull;
        a[3] = a[4] = a[5] = a[6] = a[7] = 0ull;
    }
}

// One block per chunk: chunk c covers particles [chunks[c].y, min(chunks[c].y
// + kSegChunk, part_off[s + 1])) of system s = chunks[c].x.  The chunk's
// coordinates are read as one flat run of doubles (coalesced).
template <int DIM>
__global__ void __launch_bounds__(kSegThreads)
k_seg_bbox_chunks(const double* __restrict__ pos, const double* __restrict__ mass,
                  const int64_t* __restrict__ part_off, const int2* __restrict__ chunks,
                  uint64_t* __restrict__ acc, unsigned* __restrict__ err)
{
    const int2 ch = chunks[blockIdx.x];
    const int s = ch.x;
    const int64_t p0 = ch.y, p1 = min(p0 + (int64_t)kSegChunk, part_off[s + 1]);
    const uint64_t* __restrict__ pb = reinterpret_cast<const uint64_t*>(pos);
    const uint64_t* __restrict__ mb = reinterpret_cast<const uint64_t*>(mass);
    uint64_t v[7] = {~0ull, ~0ull, ~0ull, 0ull, 0ull, 0ull, 0ull};
    bool bad = false, mdiff = false;
    for (int64_t j = p0 * DIM + threadIdx.x; j < p1 * DIM; j += blockDim.x) {
        const uint64_t x = __ldg(pb + j);
        const int d = (int)(j % DIM);
        bad |= !finite_bits(x);
        const uint64_t k = ord_key(x);
        v[d] = k < v[d] ? k : v[d];
        v[3 + d] = k > v[3 + d] ? k : v[3 + d];
    }
    const uint64_t m0 = __ldg(mb + part_off[s]);
    for (int64_t i = p0 + threadIdx.x; i < p1; i += blockDim.x) {
        const uint64_t x = __ldg(mb + i);
        bad |= !finite_bits(x);
        const uint64_t am = x & 0x7FFFFFFFFFFFFFFFull;
        v[6] = am > v[6] ? am : v[6];
        mdiff |= x != m0;
    }
    __shared__ uint64_t red[kSegThreads / 32][7];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 7; k++) {
        for (int o = 16; o > 0; o >>= 1) {
            const uint64_t y = __shfl_down_sync(0xffffffffu, v[k], o);
            v[k] = k < 3 ? (y < v[k] ? y : v[k]) : (y > v[k] ? y : v[k]);
        }
        if (lane == 0) red[warp][k] = v[k];
    }
    if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(err, kErrNonFinite);
    mdiff = __syncthreads_or(mdiff);
    if (threadIdx.x < 7) {
        const int k = threadIdx.x;
        uint64_t r = red[0][k];
        for (int w = 1; w < kSegThreads / 32; w++)
            r = k < 3 ? (red[w][k] < r ? red[w][k] : r) : (red[w][k] > r ? red[w][k] : r);
        unsigned long long* a = reinterpret_cast<unsigned long long*>(acc + kSegAcc * s + k);
        if (k < 3) {
            if (k < DIM) atomicMin(a, (unsigned long long)r);
        } else if (k < 6) {
            if (k - 3 < DIM) atomicMax(a, (unsigned long long)r);
        } else {
            atomicMax(a, (unsigned long long)r);
        }
    }
    if (threadIdx.x == 0 && mdiff)
        atomicOr(reinterpret_cast<unsigned long long*>(acc + kSegAcc * s + 7), 1ull);
}

// Per system: the box from the accumulators, the Morton quantiser's data
// (the same arithmetic as the single-tree k_bbox / k_morton) and the
// float-float frame.
__global__ void k_seg_box_finish(const uint64_t* __restrict__ acc, const double* __restrict__ mass,
                                 const int64_t* __restrict__ part_off, int dim, int64_t ns,
                                 double* __restrict__ box, FastFrame* __restrict__ frames)
{
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < ns;
         s += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t* a = acc + kSegAcc * s;
        double* bx = box + kSegBox * s;
        bool degenerate = false;
        for (int d = 0; d < 3; d++) {
            double lo = 0.0, hi = 0.0, ext = 1.0, rcp = 1.0;
            if (d < dim) {
                lo = __longlong_as_double((long long)ord_inv(a[d]));
                hi = __longlong_as_double((long long)ord_inv(a[3 + d]));
                const double e = __dsub_rn(hi, lo);
                ext = e <= 0 ? 1.0 : e;
                degenerate |= e <= 0;
                rcp = __drcp_rn(ext);
            }
            bx[d] = lo;
            bx[3 + d] = hi;
            bx[8 + d] = rcp;
            bx[12 + d] = ext;
        }
        bx[6] = __longlong_as_double((long long)a[6]);
        const double m0 = mass[part_off[s]];
        const bool unit = !(a[7] & 1ull) && m0 > 0.0 && isfinite(m0);
        bx[7] = unit ? 1.0 : 0.0;
        bx[11] = degenerate ? 1.0 : 0.0;
        FastFrame f;
        frame_from_box(bx, dim, &f);
        frame_unit_mass(bx[6], unit, &f);
        frames[s] = f;
    }
}

// Morton keys, each particle in its own system's box (sys_of: the system of
// every particle; input and sorted order share the systems' ranges).
template <int DIM>
__global__ void k_seg_morton(const double* __restrict__ pos, int64_t n,
                             const int32_t* __restrict__ sys_of, const double* __restrict__ box,
                             uint64_t* __restrict__ keys, int32_t* __restrict__ idx)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double* bx = box + kSegBox * sys_of[i];
        uint64_t c[3] = {0, 0, 0};
        if (bx[11] == 0.0) {   // division-free quantiser
#pragma unroll
            for (int d = 0; d < DIM; d++)
                c[d] = quantise_rcp(pos[DIM * i + d], bx[d], bx[12 + d], bx[8 + d]);
        } else {
#pragma unroll
            for (int d = 0; d < DIM; d++)
                c[d] = quantise(pos[DIM * i + d], bx[d], bx[12 + d],
                                __dsub_rn(bx[3 + d], bx[d]) <= 0 ? 0.5 : 0.0);
        }
        keys[i] = DIM == 3 ? morton3(c[0], c[1], c[2]) : morton2(c[0], c[1]);
        idx[i] = (int32_t)i;
    }
}

// The system of every particle and of every node (once per layout).
__global__ void __launch_bounds__(kSegThreads)
k_seg_owner(const int64_t* __restrict__ part_off, const int64_t* __restrict__ node_off,
            int32_t* __restrict__ sys_of, int32_t* __restrict__ node_sys)
{
    const int s = blockIdx.x;
    for (int64_t i = part_off[s] + threadIdx.x; i < part_off[s + 1]; i += blockDim.x)
        sys_of[i] = s;
    for (int64_t k = node_off[s] + threadIdx.x; k < node_off[s + 1]; k += blockDim.x)
        node_sys[k] = s;
}

__global__ void k_seg_key2(const int32_t* __restrict__ perm, const int32_t* __restrict__ sys_of,
                           int64_t n, uint64_t* __restrict__ key2)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        key2[i] = (uint64_t)sys_of[perm[i]];
}

// Systems marked in `keep` reuse the permutation given by the caller (a
// refit: their Morton order and topology are frozen, node boxes and moments
// are recomputed from the new positions); the others keep the fresh sort.
__global__ void k_seg_keep_perm(int64_t n, const int32_t* __restrict__ sys_of,
                                const uint8_t* __restrict__ keep,
                                const int32_t* __restrict__ perm_in, int32_t* __restrict__ perm)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        if (keep[sys_of[i]]) perm[i] = perm_in[i];
}

// should_refit_vs_rebuild (bhut/tree/refit.py:236-249) per system: flag[s]
// = 1 when a particle of system s lies beyond 1.1 x the root half-size from
// the root centre (roots: 4 doubles per system, centre and half-size of the
// root at the system's last rebuild) along some axis.
__global__ void k_seg_outside(const double* __restrict__ pos, const int64_t* __restrict__ off,
                              const double* __restrict__ roots, int dim,
                              uint8_t* __restrict__ flag)
{
    const int s = blockIdx.x;
    const double* r = roots + 4 * s;
    const double lim = __dmul_rn(1.1, r[3]);
    bool out = false;
    for (int64_t i = off[s] + threadIdx.x; i < off[s + 1]; i += blockDim.x) {
        double mx = fabs(__dsub_rn(pos[i * dim], r[0]));
        for (int d = 1; d < dim; d++) {
            const double v = fabs(__dsub_rn(pos[i * dim + d], r[d]));
            mx = v > mx ? v : mx;
        }
        out |= (mx > lim) || !(mx == mx);
    }
    out = __syncthreads_or(out);
    if (threadIdx.x == 0) flag[s] = out ? 1 : 0;
}

// The same test on the device inside a solve: a system asked to keep its
// order (keep[s] = 1) that has a particle beyond 1.1 x its stored root box is
// rebuilt instead (keep[s] <- 0, forced[s] += 1).  Per particle, the finding
// goes to flag bit 1 of the system's accumulators; k_seg_keep_finish applies
// it per system.
__global__ void k_seg_keep_outside(const double* __restrict__ pos, int64_t n, int dim,
                                   const int32_t* __restrict__ sys_of,
                                   const double* __restrict__ roots,
                                   const uint8_t* __restrict__ keep, uint64_t* __restrict__ acc)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int s = sys_of[i];
        if (!keep[s]) continue;
        const double* r = roots + 4 * s;
        const double lim = __dmul_rn(1.1, r[3]);
        double mx = fabs(__dsub_rn(pos[i * dim], r[0]));
        for (int d = 1; d < dim; d++) {
            const double v = fabs(__dsub_rn(pos[i * dim + d], r[d]));
            mx = v > mx ? v : mx;
        }
        if ((mx > lim) || !(mx == mx)) {
            unsigned long long* f = reinterpret_cast<unsigned long long*>(acc + kSegAcc * s + 7);
            if (!(*f & 2ull)) atomicOr(f, 2ull);
        }
    }
}

__global__ void k_seg_keep_finish(const uint64_t* __restrict__ acc, int64_t ns,
                                  uint8_t* __restrict__ keep, int32_t* __restrict__ forced)
{
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < ns;
         s += (int64_t)gridDim.x * blockDim.x) {
        if (keep[s] && (acc[kSegAcc * s + 7] & 2ull)) {
            keep[s] = 0;
            forced[s] += 1;
        }
    }
}

// Root boxes of the systems rebuilt by this solve (keep == NULL: all).
__global__ void k_seg_roots_update(const int64_t* __restrict__ node_off,
                                   const double* __restrict__ center,
                                   const double* __restrict__ half, int dim, int64_t ns,
                                   const uint8_t* __restrict__ keep, double* __restrict__ roots)
{
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < ns;
         s += (int64_t)gridDim.x * blockDim.x) {
        if (keep && keep[s]) continue;
        const int64_t r = node_off[s];
        for (int d = 0; d < 3; d++) roots[4 * s + d] = d < dim ? center[r * dim + d] : 0.0;
        roots[4 * s + 3] = half[r];
    }
}

// Root centre and half-size of every system from the last solve.
__global__ void k_seg_roots(const int64_t* __restrict__ node_off, const double* __restrict__ center,
                            const double* __restrict__ half, int dim, int64_t ns,
                            double* __restrict__ roots)
{
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < ns;
         s += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = node_off[s];
        for (int d = 0; d < 3; d++) roots[4 * s + d] = d < dim ? center[r * dim + d] : 0.0;
        roots[4 * s + 3] = half[r];
    }
}

// Leapfrog kick and drift: v += kick * a, then x += drift * v.
__global__ void k_leapfrog(double* __restrict__ pos, double* __restrict__ vel,
                           const double* __restrict__ acc, int64_t n, double kick, double drift)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double v = __fma_rn(kick, acc[i], vel[i]);
        vel[i] = v;
        if (drift != 0.0) pos[i] = __fma_rn(drift, v, pos[i]);
    }
}

// One block per system.  Thread 0 builds the per-depth tables of the
// closed form (see k_topology in build.cu) in shared memory; the block then
// walks that system's BFS slots.
__global__ void __launch_bounds__(kSegThreads)
k_seg_topology(const int64_t* __restrict__ part_off, const int64_t* __restrict__ node_off,
               const int64_t* __restrict__ leaf_off, int leaf_size,
               int32_t* __restrict__ first_child, int32_t* __restrict__ start,
               int32_t* __restrict__ count, int32_t* __restrict__ parent,
               int32_t* __restrict__ leaf_list, unsigned* __restrict__ err)
{
    const int s = blockIdx.x;
    const int64_t n = part_off[s + 1] - part_off[s];
    const int64_t L = leaf_size;
    __shared__ int64_t cnt_lo[kMaxDepth];
    __shared__ int64_t internal[kMaxDepth][2];
    __shared__ int depth_s;
    __shared__ unsigned leaf_ctr;
    if (threadIdx.x == 0) {
        int depth = 0;
        while (((n + (1ll << depth) - 1) >> depth) > L && depth < kMaxDepth - 2) depth++;
        depth_s = depth;
        for (int d = 0; d <= depth + 1; d++) cnt_lo[d] = n >> d;
        for (int d = depth + 1; d >= 0; d--) {
            for (int v = 0; v < 2; v++) {
                const int64_t c = cnt_lo[d] + v;
                if (c <= L) { internal[d][v] = 0; continue; }
                const int64_t h = c / 2, r = c - h, lo = cnt_lo[d + 1];
                internal[d][v] = 1 + internal[d + 1][h - lo] + internal[d + 1][r - lo];
            }
        }
        leaf_ctr = 0;
    }
    __syncthreads();
    const int depth = depth_s;
    const int64_t nodes = node_off[s + 1] - node_off[s];
    const int64_t leaves = leaf_off[s + 1] - leaf_off[s];
    const int64_t slots = (2ll << depth) - 1;
    const int64_t nb = node_off[s], pb = part_off[s];
    for (int64_t slot = threadIdx.x; slot < slots; slot += blockDim.x) {
        const int d = 63 - __clzll((unsigned long long)(slot + 1));
        const int64_t j = slot + 1 - (1ll << d);
        int64_t c = n, st = 0, k = 0, id = 0, par = -1;
        bool exists = true;
        for (int t = 0; t < d; t++) {
            if (c <= L) { exists = false; break; }
            const int bit = (int)((j >> (d - 1 - t)) & 1);
            const int64_t half = c / 2, rc = c - half;
            par = id;
            if (bit == 0) {
                id = 2 * k + 1;
                k = k + 1 + internal[t + 1][rc - cnt_lo[t + 1]];
                c = half;
            } else {
                id = 2 * k + 2;
                k = k + 1;
                st += half;
                c = rc;
            }
        }
        if (!exists) continue;
        if (id >= nodes || st + c > n) { atomicOr(err, kErrBadNode); continue; }
        start[nb + id] = (int32_t)(pb + st);
        count[nb + id] = (int32_t)c;
        parent[nb + id] = par < 0 ? -1 : (int32_t)(nb + par);
        if (c <= L) {
            first_child[nb + id] = -1;
            const unsigned li = atomicAdd(&leaf_ctr, 1u);
            if (li < leaves) leaf_list[leaf_off[s] + li] = (int32_t)(nb + id);
            else atomicOr(err, kErrBadNode);
        } else {
            first_child[nb + id] = (int32_t)(nb + 2 * k + 1);
        }
    }
}

// Float-float copies of every particle and node in its system's frame.
__global__ void k_seg_ff_particles(TreeDev t, const int32_t* __restrict__ sys_of,
                                   const FastFrame* __restrict__ frames, float4* __restrict__ ph,
                                   float4* __restrict__ pl)
{
    const int dim = t.dim;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < t.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const FastFrame& f = frames[sys_of[i]];
        float4 h, l;
        split_grid(__dmul_rn(__dsub_rn(t.sx[i], f.c[0]), f.s), h.x, l.x);
        split_grid(__dmul_rn(__dsub_rn(t.sy[i], f.c[1]), f.s), h.y, l.y);
        if (dim == 3) split_grid(__dmul_rn(__dsub_rn(t.sz[i], f.c[2]), f.s), h.z, l.z);
        else h.z = l.z = 0.0f;
        if (f.unit) { h.w = 1.0f; l.w = 0.0f; }   // every mass is m0: exactly 1 in units of m0
        else split_plain(__dmul_rn(t.sm[i], f.ms), h.w, l.w);
        ph[i] = h;
        pl[i] = l;
    }
}

__global__ void k_seg_ff_nodes(TreeDev t, const int32_t* __restrict__ node_sys,
                               const FastFrame* __restrict__ frames,
                               const double* __restrict__ center, float4* __restrict__ nh,
                               float4* __restrict__ nl, float* __restrict__ nsize,
                               float* __restrict__ ndelta, const double* __restrict__ quad,
                               float4* __restrict__ nq0, float2* __restrict__ nq1,
                               int4* __restrict__ nhdr)
{
    const int dim = t.dim;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < t.m;
         k += (int64_t)gridDim.x * blockDim.x) {
        const FastFrame& f = frames[node_sys[k]];
        const NodeCM c = t.cm[k];
        float4 h, l;
        split_grid(__dmul_rn(__dsub_rn(c.x, f.c[0]), f.s), h.x, l.x);
        split_grid(__dmul_rn(__dsub_rn(c.y, f.c[1]), f.s), h.y, l.y);
        if (dim == 3) split_grid(__dmul_rn(__dsub_rn(c.z, f.c[2]), f.s), h.z, l.z);
        else h.z = l.z = 0.0f;
        split_plain(__dmul_rn(c.w, f.ms), h.w, l.w);
        nh[k] = h;
        nl[k] = l;
        nsize[k] = __double2float_rn(__dmul_rn(t.size[k], f.s));
        double dd = 0.0;
        for (int d = 0; d < dim; d++) {
            const double cc = d == 0 ? c.x : (d == 1 ? c.y : c.z);
            const double v = cc - center[k * dim + d];
            dd += v * v;
        }
        ndelta[k] = __double2float_ru(sqrt(dd) * f.s);
        // header: leaf (-1, start, count, mass != 0); internal (first child,
        // size, |com - centre| as float bits, mass != 0)
        const int fc = t.first_child[k];
        nhdr[k] = fc < 0 ? make_int4(fc, t.start[k], t.count[k], c.w != 0.0)
                         : make_int4(fc, __float_as_int(nsize[k]), __float_as_int(ndelta[k]),
                                     c.w != 0.0);
        if (quad) {   // mass x length^2: scale by ms s^2
            const double qs = f.ms * f.s * f.s;
            const double* q = quad + 6 * k;
            nq0[k] = make_float4((float)(q[0] * qs), (float)(q[1] * qs), (float)(q[2] * qs),
                                 (float)(q[3] * qs));
            nq1[k] = make_float2((float)(q[4] * qs), (float)(q[5] * qs));
        }
    }
}

// ---------------------------------------------------------------------------
// persistent traversal
// ---------------------------------------------------------------------------
struct BatchDev {
    TreeDev t;                    // global forest (node ids, particles)
    const int64_t* part_off;
    const int64_t* node_off;
    const FastFrame* frames;
    const float4* ph;
    const float4* pl;
    const float4* nh;
    const float4* nl;
    const float* nsize;
    const float* ndelta;
    const float4* nq0;            // quadrupoles (FP32 form); NULL: monopoles
    const float2* nq1;
    const int4* nhdr;             // (first_child, start, count, mass != 0)
};

struct BatchArgs {
    const int2* tasks;            // (system, chunk), heaviest systems first
    int ntasks;
    unsigned* counter;            // task ticket counter (zeroed before launch)
    double theta, eps, G;
    int mac;
    double* out;                  // (N_total, dim), input order
    unsigned* err;
    unsigned long long* stats;
};

// The warp's traversal stack of (node, lane mask) entries, two placements:
//  STK 0: in shared memory, lane 0 writes, every lane reads (one __syncwarp
//         per pop and per push);
//  STK 1: in registers, entry j held by lane j % 32 in register j / 32;
//         a pop is two shuffles from the owning lane, a push a predicated
//         register write; no shared memory, no __syncwarp.
// Entries are warp-uniform, so every lane keeps the same depth `sp`.
template <int STK> struct WarpStack;

template <> struct WarpStack<0> {
    int2* s;
    int sp = 0, lane;
    __device__ WarpStack(int2* s_, int lane_) : s(s_), lane(lane_) {}
    __device__ void init(int node, unsigned mask)
    {
        if (lane == 0) s[0] = make_int2(node, (int)mask);
        sp = 1;
        __syncwarp();
    }
    __device__ bool empty() const { return sp == 0; }
    __device__ int2 pop()
    {
        const int2 e = s[--sp];
        __syncwarp();
        return e;
    }
    __device__ bool push2(int fc, unsigned m)
    {
        if (sp + 2 > kStackDepth) return false;
        if (lane == 0) {
            s[sp] = make_int2(fc, (int)m);
            s[sp + 1] = make_int2(fc + 1, (int)m);
        }
        sp += 2;
        __syncwarp();
        return true;
    }
};

template <> struct WarpStack<1> {
    static_assert(kStackDepth <= 2 * kWarp, "register stack holds two entries per lane");
    int n0 = 0, m0 = 0, n1 = 0, m1 = 0;
    int sp = 0, lane;
    __device__ WarpStack(int2*, int lane_) : lane(lane_) {}
    __device__ void put(int j, int node, int mask)
    {
        if (lane == (j & 31)) {
            if (j < kWarp) { n0 = node; m0 = mask; }
            else { n1 = node; m1 = mask; }
        }
    }
    __device__ void init(int node, unsigned mask)
    {
        put(0, node, (int)mask);
        sp = 1;
    }
    __device__ bool empty() const { return sp == 0; }
    __device__ int2 pop()
    {
        --sp;
        const bool hi = sp >= kWarp;
        const int node = __shfl_sync(0xffffffffu, hi ? n1 : n0, sp & 31);
        const int mask = __shfl_sync(0xffffffffu, hi ? m1 : m0, sp & 31);
        return make_int2(node, mask);
    }
    __device__ bool push2(int fc, unsigned m)
    {
        if (sp + 2 > kStackDepth) return false;
        put(sp, fc, (int)m);
        put(sp + 1, fc + 1, (int)m);
        sp += 2;
        return true;
    }
};

template <int DIM, bool FP32, int TPW, int STK>
__global__ void __launch_bounds__(kBatchThreads)
k_batch_traverse(BatchDev b, BatchArgs a)
{
    constexpr int LPT = kWarp / TPW;            // lanes per target
    __shared__ int2 stack[STK == 0 ? kBatchWarps : 1][kStackDepth];
    __shared__ float4 sh[kBatchWarps][kWarp], sl[kBatchWarps][kWarp];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int sub = lane % LPT;
    const unsigned FULL = 0xffffffffu;
    const TreeDev& t = b.t;
    const float theta_f = (float)a.theta;
    const double eps2 = __dmul_rn(a.eps, a.eps);
    unsigned long long tot[5] = {0, 0, 0, 0, 0};

    while (true) {
        int task = 0;
        if (lane == 0) task = (int)atomicAdd(a.counter, 1u);
        task = __shfl_sync(FULL, task, 0);
        if (task >= a.ntasks) break;
        const int2 tk = a.tasks[task];
        const int sys = tk.x;
        const int64_t p1 = b.part_off[sys + 1];
        const int64_t i = b.part_off[sys] + (int64_t)tk.y * TPW + lane / LPT;
        const bool valid = i < p1;
        const FastFrame fr = b.frames[sys];
        const int root = (int)b.node_off[sys];
        const double es = __dmul_rn(a.eps, fr.s);
        const double e2 = __dmul_rn(es, es);
        const float e2h = __double2float_rn(e2);
        const float e2l = __double2float_rn(__dsub_rn(e2, (double)e2h));
        // softening large enough that no pair needs the small-R test
        const bool soft = FP32 ? e2h >= 0x1p-126f : e2h >= 2.0f * kTinyR;

        float Th[3] = {0.f, 0.f, 0.f}, Tl[3] = {0.f, 0.f, 0.f};
        double x = 0.0, y = 0.0, z = 0.0;
        if (valid) {
            const float4 h = b.ph[i], l = b.pl[i];
            Th[0] = h.x; Th[1] = h.y; Th[2] = h.z;
            Tl[0] = l.x; Tl[1] = l.y; Tl[2] = l.z;
            if (!FP32) {
                x = t.sx[i];
                y = t.sy[i];
                z = DIM == 3 ? t.sz[i] : 0.0;
            }
        }
        const TargetF32x2 tx = target_f32x2(Th, Tl);
        const bool unit = fr.unit != 0;   // every particle mass of this system exactly 1
        float ah[3] = {0.f, 0.f, 0.f}, al[3] = {0.f, 0.f, 0.f};   // ff sum, or (sum, Kahan comp)
        double a64[3] = {0.0, 0.0, 0.0};
        unsigned cnt[5] = {0, 0, 0, 0, 0};
        bool overflow = false;

        const unsigned live = __ballot_sync(FULL, valid);
        WarpStack<STK> st(stack[STK == 0 ? w : 0], lane);
        st.init(root, live);
        while (!st.empty()) {
            const int2 e = st.pop();
            const int node = e.x;
            const bool act = ((unsigned)e.y >> lane) & 1u;
            cnt[2] += act && sub == 0;
            const int4 hd = b.nhdr[node];   // (first_child, start, count, mass != 0)
            if (!hd.w) continue;
            const int fc = hd.x;
            if (fc < 0) {
                const int s0 = hd.y, c = hd.z;
                for (int bb = 0; bb < c; bb += kWarp) {
                    const int jj = bb + lane;
                    if (jj < c) {
                        sh[w][lane] = b.ph[s0 + jj];
                        sl[w][lane] = b.pl[s0 + jj];
                    }
                    __syncwarp();
                    const int cn = min(kWarp, c - bb);
                    if (act && sub == 0) cnt[0] += cn - (i >= s0 + bb && i < s0 + bb + cn);
                    if (!FP32 && LPT == 1 && soft) {   // as the single-tree walk
                        if (unit)
                            leaf_block_soft<DIM, true>((unsigned)e.y, lane, Th, Tl, sh[w], sl[w],
                                                       cn, e2h, e2l, ah, al);
                        else
                            leaf_block_soft<DIM, false>((unsigned)e.y, lane, Th, Tl, sh[w], sl[w],
                                                        cn, e2h, e2l, ah, al);
                    } else if (act) {
                        if (FP32) {   // <= 32 terms in FP32, then one Kahan step
                            float2 pxy = make_float2(0.f, 0.f);
                            float pz = 0.f;
                            if (soft && unit) {
#pragma unroll 8
                                for (int q = sub; q < cn; q += LPT)
                                    pair_f32_partial2<DIM, false, true>(tx, sh[w][q], sl[w][q],
                                                                        e2h, pxy, pz);
                            } else if (soft) {
#pragma unroll 8
                                for (int q = sub; q < cn; q += LPT)
                                    pair_f32_partial2<DIM, false, false>(tx, sh[w][q], sl[w][q],
                                                                         e2h, pxy, pz);
                            } else {
#pragma unroll 8
                                for (int q = sub; q < cn; q += LPT)
                                    pair_f32_partial2<DIM, true, false>(tx, sh[w][q], sl[w][q],
                                                                        e2h, pxy, pz);
                            }
                            const float part[3] = {pxy.x, pxy.y, pz};
                            kahan_add_f32<DIM>(part, ah, al);
                        } else {
                            unsigned fb = 0;   // pairs left to FP64, taken after the loop
                            if (soft && unit) {
                                for (int q = sub; q < cn; q += LPT)
                                    pair_ff_soft<DIM, true>(Th, Tl, sh[w][q], sl[w][q], e2h, e2l,
                                                            ah, al);
                            } else if (soft) {
                                for (int q = sub; q < cn; q += LPT)
                                    pair_ff_soft<DIM, false>(Th, Tl, sh[w][q], sl[w][q], e2h, e2l,
                                                             ah, al);
                            } else {
                                for (int q = sub; q < cn; q += LPT)
                                    fb |= (unsigned)!pair_ff<DIM, false>(Th, Tl, sh[w][q],
                                                                         sl[w][q], e2h, e2l, ah,
                                                                         al) << q;
                            }
                            while (fb) {
                                const int gi = s0 + bb + __ffs(fb) - 1;
                                fb &= fb - 1;
                                pair_fp64<DIM>(x, y, z, t.sx[gi], t.sy[gi],
                                               DIM == 3 ? t.sz[gi] : 0.0, t.sm[gi], eps2, a64);
                                cnt[4]++;
                            }
                        }
                    }
                    __syncwarp();
                }
                if (!FP32 && act) {
#pragma unroll
                    for (int k = 0; k < DIM; k++) {
                        const float hs = __fadd_rn(ah[k], al[k]);
                        al[k] = __fsub_rn(al[k], __fsub_rn(hs, ah[k]));
                        ah[k] = hs;
                    }
                }
            } else {
                bool open = false;
                float4 nhv = make_float4(0.f, 0.f, 0.f, 0.f), nlv = nhv;
                if (act) {
                    nhv = b.nh[node];
                    if (!FP32) nlv = b.nl[node];
                    float d2 = 0.0f;
#pragma unroll
                    for (int k = 0; k < DIM; k++) {
                        // FP32 form: hi coordinates only (exact differences),
                        // as the single-tree FP32 walk
                        const float d = FP32 ? __fsub_rn(comp(nhv, k), Th[k])
                                             : __fadd_rn(__fsub_rn(comp(nhv, k), Th[k]),
                                                         __fsub_rn(comp(nlv, k), Tl[k]));
                        d2 = fmaf(d, d, d2);
                    }
                    const float dist = d2 > 0.0f ? d2 * rsqrtf(d2) : 0.0f;
                    const float size_f = __int_as_float(hd.y);
                    if (FP32) {
                        open = a.mac == 1 ? size_f >= theta_f * (dist - __int_as_float(hd.z))
                                          : (dist == 0.0f || size_f >= theta_f * dist);
                    } else {
                        const float td = theta_f * dist;
                        const float band = theta_f * fmaf(kBandRel, dist, 2.0f * kBandAbs);
                        if (size_f >= td + band) open = true;
                        else if (size_f < td - band) open = false;
                        else {
                            open = open_exact64<DIM>(x, y, z, t.cm[node], t.size[node], a.theta);
                            cnt[3]++;
                        }
                    }
                }
                const unsigned omask = __ballot_sync(FULL, act && open);
                if (act && !open && sub == 0) {
                    if (FP32) {
                        nlv = b.nl[node];
                        if (b.nq0)
                            node_quad_f32<DIM>(Th, Tl, nhv, nlv, b.nq0[node], b.nq1[node], e2h,
                                               ah, al);
                        else
                            pair_f32<DIM>(Th, Tl, nhv, nlv, e2h, ah, al);
                    } else if (soft) {
                        pair_ff_soft<DIM, false>(Th, Tl, nhv, nlv, e2h, e2l, ah, al);
                    } else if (!pair_ff<DIM, false>(Th, Tl, nhv, nlv, e2h, e2l, ah, al)) {
                        const NodeCM cm = t.cm[node];
                        pair_fp64<DIM>(x, y, z, cm.x, cm.y, cm.z, cm.w, eps2, a64);
                        cnt[4]++;
                    }
                    cnt[1]++;
                }
                if (omask && !st.push2(fc, omask)) {
                    overflow = true;
                    break;
                }
            }
        }
        if (overflow && lane == 0) atomicOr(a.err, kErrStackOverflow);
        // fold the lanes that share a target
        if (LPT == 2) {
#pragma unroll
            for (int k = 0; k < DIM; k++) {
                const float oh = __shfl_down_sync(FULL, ah[k], 1);
                const float ol = __shfl_down_sync(FULL, al[k], 1);
                const double o64 = __shfl_down_sync(FULL, a64[k], 1);
                if (FP32) {
                    ah[k] = __fadd_rn(ah[k], oh);
                    al[k] = __fadd_rn(al[k], ol);
                } else {
                    const float s2 = __fadd_rn(ah[k], oh);
                    al[k] = __fadd_rn(__fadd_rn(al[k], ol), two_sum_err(ah[k], oh, s2));
                    ah[k] = s2;
                }
                a64[k] = a64[k] + o64;
            }
        }
        for (int k = 0; k < 5; k++) tot[k] += cnt[k];
        if (valid && sub == 0) {
            const double conv = __dmul_rn(fr.conv, a.G);
            const int64_t o = t.perm[i];
#pragma unroll
            for (int k = 0; k < DIM; k++) {
                const double v = FP32 ? __dsub_rn((double)ah[k], (double)al[k])
                                      : __dadd_rn((double)ah[k], (double)al[k]);
                a.out[o * DIM + k] = __dadd_rn(__dmul_rn(v, conv), __dmul_rn(a64[k], a.G));
            }
        }
    }
    if (a.stats) {
        for (int k = 0; k < 5; k++) {
            unsigned long long v = tot[k];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
            if (lane == 0 && v) atomicAdd(&a.stats[k], v);
        }
    }
}

// Persistent grid: as many blocks as fit on the GPU at once for this
// variant (its register count decides: 5 to 8 blocks of 128 per SM).
template <int DIM, bool FP32, int TPW, int STK>
unsigned persistent_grid()
{
    static unsigned grid = 0;
    if (grid == 0) {
        int per_sm = 0, dev = 0, sms = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &per_sm, k_batch_traverse<DIM, FP32, TPW, STK>, kBatchThreads, 0) != cudaSuccess ||
            per_sm <= 0)
            per_sm = 6;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            sms <= 0)
            sms = 152;
        cudaGetLastError();
        grid = (unsigned)(per_sm * sms);
    }
    return grid;
}

// Runs the occupancy query of the configured variant once, before any
// stream capture.
template <int DIM, bool FP32, int TPW>
void prime_grid_of(int stk)
{
    if (stk == BHUT_STACK_REGISTERS) persistent_grid<DIM, FP32, TPW, 1>();
    else persistent_grid<DIM, FP32, TPW, 0>();
}

template <int DIM, bool FP32, int TPW>
void launch_batch_traverse(int stk, cudaStream_t s, const BatchDev& bd, const BatchArgs& a)
{
    if (stk == BHUT_STACK_REGISTERS)
        k_batch_traverse<DIM, FP32, TPW, 1>
            <<<persistent_grid<DIM, FP32, TPW, 1>(), kBatchThreads, 0, s>>>(bd, a);
    else
        k_batch_traverse<DIM, FP32, TPW, 0>
            <<<persistent_grid<DIM, FP32, TPW, 0>(), kBatchThreads, 0, s>>>(bd, a);
}

inline size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

// ---------------------------------------------------------------------------
// handle
// ---------------------------------------------------------------------------
struct BufB {
    void* p = nullptr;
    size_t bytes = 0;
    int ensure(size_t need, cudaStream_t s)
    {
        if (need <= bytes && p) return kOk;
        if (p) { cudaFreeAsync(p, s); p = nullptr; bytes = 0; }
        cudaError_t e = cudaMallocAsync(&p, need < 256 ? 256 : need, s);
        if (e != cudaSuccess) { p = nullptr; return cuda_status(e, "cudaMallocAsync"); }
        bytes = need < 256 ? 256 : need;
        return kOk;
    }
    void release(cudaStream_t s) { if (p) cudaFreeAsync(p, s); p = nullptr; bytes = 0; }
    template <class T> T* as() const { return (T*)p; }
};

struct bhut_batch {
    int dim = 3, leaf = 32, form = BHUT_FORM_FP32, mac = 0, tpw = 32;
    int multipole = BHUT_MULTIPOLE_MONO;
    int stack = BHUT_STACK_SHARED;
    bool refit_rule = false;        // refit-vs-rebuild test inside the solve
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int64_t nsys = 0, ntot = 0, mtot = 0, ltot = 0;
    std::vector<int64_t> part_off, node_off, leaf_off;
    std::vector<int2> tasks;
    bool layout_valid = false, built = false, topo_valid = false;
    BufB pos, mass, d_part_off, d_node_off, d_leaf_off, d_tasks, keys, perm, sys_of, key2,
        sx, sy, sz, sm, cm, size, center, half, lo, hi, first_child, start, count, parent,
        leaf_list, arrive, sort_scratch, box, frames, ph, pl, nh, nl, nsize, ndelta, counter,
        err, stats, out, keep, perm_in, quad, nq0, nq1, nhdr, roots, forced, frontier,
        node_sys, acc, d_chunks;
    int64_t nchunks = 0;
    bool keep_active = false;
    unsigned long long last_stats[5] = {0, 0, 0, 0, 0};
    cudaGraphExec_t graph = nullptr;
    bool use_graph = false;
    cudaEvent_t ev_trav[2] = {nullptr, nullptr};   // around the traversal (graph nodes too)
    double g_theta = -1, g_eps = -1, g_G = 0;
    double* g_out = nullptr;

    void release_all()
    {
        for (BufB* x : {&pos, &mass, &d_part_off, &d_node_off, &d_leaf_off, &d_tasks, &keys, &perm,
                        &sys_of, &key2, &sx, &sy, &sz, &sm, &cm, &size, &center, &half, &lo, &hi,
                        &first_child, &start, &count, &parent, &leaf_list, &arrive,
                        &sort_scratch, &box, &frames, &ph, &pl, &nh, &nl, &nsize, &ndelta,
                        &counter, &err, &stats, &out, &keep, &perm_in, &quad, &nq0, &nq1, &nhdr,
                        &roots, &forced, &frontier, &node_sys, &acc, &d_chunks})
            x->release(stream);
    }

    TreeDev dev() const
    {
        TreeDev t;
        t.dim = dim; t.leaf_size = leaf; t.n = ntot; t.m = mtot;
        t.sx = sx.as<double>(); t.sy = sy.as<double>(); t.sz = sz.as<double>();
        t.sm = sm.as<double>(); t.perm = perm.as<int32_t>(); t.cm = cm.as<NodeCM>();
        t.size = size.as<double>(); t.first_child = first_child.as<int32_t>();
        t.start = start.as<int32_t>(); t.count = count.as<int32_t>();
        return t;
    }
};

namespace {

void drop_graph(bhut_batch* b)
{
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
}

// Task list: (system, chunk of tpw targets), heaviest systems first so that
// the queue drains evenly.
int plan_tasks(bhut_batch* b)
{
    std::vector<std::pair<int64_t, int>> order;
    for (int64_t s = 0; s < b->nsys; s++)
        order.push_back({b->part_off[s + 1] - b->part_off[s], (int)s});
    std::stable_sort(order.begin(), order.end(),
                     [](const std::pair<int64_t, int>& x, const std::pair<int64_t, int>& y) {
                         return x.first > y.first;
                     });
    b->tasks.clear();
    for (auto& o : order) {
        const int64_t chunks = (o.first + b->tpw - 1) / b->tpw;
        for (int64_t c = 0; c < chunks; c++) b->tasks.push_back(make_int2(o.second, (int)c));
    }
    BHUT_TRY(b->d_tasks.ensure(sizeof(int2) * b->tasks.size(), b->stream));
    BHUT_CUDA(cudaMemcpyAsync(b->d_tasks.p, b->tasks.data(), sizeof(int2) * b->tasks.size(),
                              cudaMemcpyHostToDevice, b->stream));
    BHUT_CUDA(cudaStreamSynchronize(b->stream));   // the host vector is reused
    return kOk;
}

// Host plan: node and leaf counts of every system, buffers, task list.
int plan_layout(bhut_batch* b, const int64_t* offsets, int64_t nsys)
{
    b->part_off.assign(offsets, offsets + nsys + 1);
    b->node_off.assign(nsys + 1, 0);
    b->leaf_off.assign(nsys + 1, 0);
    for (int64_t s = 0; s < nsys; s++) {
        const int64_t n = offsets[s + 1] - offsets[s];
        if (n <= 0) { set_error("system %lld has no particles", (long long)s); return kInvalid; }
        TopoTables tt;
        BHUT_TRY(make_topo_tables(n, b->leaf, &tt));
        b->node_off[s + 1] = b->node_off[s] + tt.num_nodes;
        b->leaf_off[s + 1] = b->leaf_off[s] + tt.num_leaves;
    }
    b->nsys = nsys;
    b->ntot = offsets[nsys];
    b->mtot = b->node_off[nsys];
    b->ltot = b->leaf_off[nsys];
    if (b->ntot > 0x7fffffffLL || b->mtot > 0x7fffffffLL) {
        set_error("batch too large: at most 2^31-1 particles and nodes");
        return kInvalid;
    }
    cudaStream_t s = b->stream;
    const size_t ntot = (size_t)b->ntot, mtot = (size_t)b->mtot;
    BHUT_TRY(b->d_part_off.ensure(sizeof(int64_t) * (nsys + 1), s));
    BHUT_TRY(b->d_node_off.ensure(sizeof(int64_t) * (nsys + 1), s));
    BHUT_TRY(b->d_leaf_off.ensure(sizeof(int64_t) * (nsys + 1), s));
    BHUT_CUDA(cudaMemcpyAsync(b->d_part_off.p, b->part_off.data(), sizeof(int64_t) * (nsys + 1),
                              cudaMemcpyHostToDevice, s));
    BHUT_CUDA(cudaMemcpyAsync(b->d_node_off.p, b->node_off.data(), sizeof(int64_t) * (nsys + 1),
                              cudaMemcpyHostToDevice, s));
    BHUT_CUDA(cudaMemcpyAsync(b->d_leaf_off.p, b->leaf_off.data(), sizeof(int64_t) * (nsys + 1),
                              cudaMemcpyHostToDevice, s));
    BHUT_TRY(plan_tasks(b));
    const int dim = b->dim;
    BHUT_TRY(b->pos.ensure(sizeof(double) * ntot * dim, s));
    BHUT_TRY(b->mass.ensure(sizeof(double) * ntot, s));
    BHUT_TRY(b->keys.ensure(sizeof(uint64_t) * ntot, s));
    BHUT_TRY(b->key2.ensure(sizeof(uint64_t) * ntot, s));
    BHUT_TRY(b->perm.ensure(sizeof(int32_t) * ntot, s));
    BHUT_TRY(b->sys_of.ensure(sizeof(int32_t) * ntot, s));
    for (BufB* x : {&b->sx, &b->sy, &b->sz, &b->sm}) BHUT_TRY(x->ensure(sizeof(double) * ntot, s));
    BHUT_TRY(b->ph.ensure(sizeof(float4) * ntot, s));
    BHUT_TRY(b->pl.ensure(sizeof(float4) * ntot, s));
    BHUT_TRY(b->out.ensure(sizeof(double) * ntot * dim, s));
    BHUT_TRY(b->cm.ensure(sizeof(NodeCM) * mtot, s));
    for (BufB* x : {&b->size, &b->half}) BHUT_TRY(x->ensure(sizeof(double) * mtot, s));
    BHUT_TRY(b->center.ensure(sizeof(double) * mtot * dim, s));
    BHUT_TRY(b->lo.ensure(sizeof(double) * mtot * 3, s));
    BHUT_TRY(b->hi.ensure(sizeof(double) * mtot * 3, s));
    for (BufB* x : {&b->first_child, &b->start, &b->count, &b->parent})
        BHUT_TRY(x->ensure(sizeof(int32_t) * mtot, s));
    BHUT_TRY(b->arrive.ensure(sizeof(unsigned) * mtot, s));
    BHUT_TRY(b->leaf_list.ensure(sizeof(int32_t) * b->ltot, s));
    BHUT_TRY(b->frontier.ensure(sizeof(int32_t) * b->ltot, s));
    BHUT_TRY(b->nh.ensure(sizeof(float4) * mtot, s));
    BHUT_TRY(b->nl.ensure(sizeof(float4) * mtot, s));
    BHUT_TRY(b->nsize.ensure(sizeof(float) * mtot, s));
    BHUT_TRY(b->ndelta.ensure(sizeof(float) * mtot, s));
    BHUT_TRY(b->quad.ensure(sizeof(double) * 6 * mtot, s));
    BHUT_TRY(b->nq0.ensure(sizeof(float4) * mtot, s));
    BHUT_TRY(b->nq1.ensure(sizeof(float2) * mtot, s));
    BHUT_TRY(b->nhdr.ensure(sizeof(int4) * mtot, s));
    BHUT_TRY(b->box.ensure(sizeof(double) * kSegBox * nsys, s));
    BHUT_TRY(b->acc.ensure(sizeof(uint64_t) * kSegAcc * nsys, s));
    BHUT_TRY(b->node_sys.ensure(sizeof(int32_t) * mtot, s));
    {   // chunks of at most kSegChunk particles, each inside one system
        std::vector<int2> ch;
        for (int64_t q = 0; q < nsys; q++)
            for (int64_t p = b->part_off[q]; p < b->part_off[q + 1]; p += kSegChunk)
                ch.push_back(make_int2((int)q, (int)p));
        b->nchunks = (int64_t)ch.size();
        BHUT_TRY(b->d_chunks.ensure(sizeof(int2) * ch.size(), s));
        BHUT_CUDA(cudaMemcpyAsync(b->d_chunks.p, ch.data(), sizeof(int2) * ch.size(),
                                  cudaMemcpyHostToDevice, s));
        BHUT_CUDA(cudaStreamSynchronize(s));   // the host vector goes out of scope
    }
    k_seg_owner<<<(unsigned)nsys, kSegThreads, 0, s>>>(b->d_part_off.as<int64_t>(),
                                                       b->d_node_off.as<int64_t>(),
                                                       b->sys_of.as<int32_t>(),
                                                       b->node_sys.as<int32_t>());
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    BHUT_TRY(b->frames.ensure(sizeof(FastFrame) * nsys, s));
    BHUT_TRY(b->sort_scratch.ensure(sort_scratch_bytes(b->ntot), s));
    BHUT_TRY(b->counter.ensure(sizeof(unsigned) * 4, s));
    BHUT_TRY(b->err.ensure(sizeof(unsigned), s));
    BHUT_TRY(b->stats.ensure(sizeof(unsigned long long) * 8, s));
    BHUT_CUDA(cudaMemsetAsync(b->err.p, 0, sizeof(unsigned), s));
    BHUT_TRY(b->keep.ensure(nsys, s));
    BHUT_TRY(b->roots.ensure(sizeof(double) * 4 * nsys, s));
    BHUT_TRY(b->forced.ensure(sizeof(int32_t) * nsys, s));
    BHUT_CUDA(cudaMemsetAsync(b->roots.p, 0, sizeof(double) * 4 * nsys, s));
    BHUT_CUDA(cudaMemsetAsync(b->forced.p, 0, sizeof(int32_t) * nsys, s));
    BHUT_TRY(b->perm_in.ensure(sizeof(int32_t) * ntot, s));
    b->keep_active = false;
    b->layout_valid = true;
    b->topo_valid = false;
    drop_graph(b);
    return kOk;
}

int bits_for(int64_t v)
{
    int b = 1;
    while (b < 62 && (1ll << b) <= v) b++;
    return b;
}

// All device work of one solve (build + traversal), stream-ordered, no host
// synchronisation: this is what a CUDA graph captures.
// Records a timing event on s.  Under stream capture a plain record only
// marks a dependency and the event is never recorded when the graph runs;
// an external record becomes a graph node that records it on every replay.
int record_timing_event(cudaEvent_t e, cudaStream_t s)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    BHUT_CUDA(cudaStreamIsCapturing(s, &cs));
    if (cs == cudaStreamCaptureStatusActive)
        BHUT_CUDA(cudaEventRecordWithFlags(e, s, cudaEventRecordExternal));
    else
        BHUT_CUDA(cudaEventRecord(e, s));
    return kOk;
}

int enqueue_solve(bhut_batch* b, double theta, double eps, double G, double* out)
{
    cudaStream_t s = b->stream;
    const int dim = b->dim;
    const int64_t ns = b->nsys, n = b->ntot;
    const unsigned gs = grid_for(ns, 128);
    k_seg_acc_init<<<gs, 128, 0, s>>>(b->acc.as<uint64_t>(), ns);
    if (dim == 3)
        k_seg_bbox_chunks<3><<<(unsigned)b->nchunks, kSegThreads, 0, s>>>(
            b->pos.as<double>(), b->mass.as<double>(), b->d_part_off.as<int64_t>(),
            b->d_chunks.as<int2>(), b->acc.as<uint64_t>(), b->err.as<unsigned>());
    else
        k_seg_bbox_chunks<2><<<(unsigned)b->nchunks, kSegThreads, 0, s>>>(
            b->pos.as<double>(), b->mass.as<double>(), b->d_part_off.as<int64_t>(),
            b->d_chunks.as<int2>(), b->acc.as<uint64_t>(), b->err.as<unsigned>());
    k_seg_box_finish<<<gs, 128, 0, s>>>(b->acc.as<uint64_t>(), b->mass.as<double>(),
                                        b->d_part_off.as<int64_t>(), dim, ns, b->box.as<double>(),
                                        b->frames.as<FastFrame>());
    if (dim == 3)
        k_seg_morton<3><<<grid_for(n, 256), 256, 0, s>>>(b->pos.as<double>(), n,
                                                         b->sys_of.as<int32_t>(),
                                                         b->box.as<double>(),
                                                         b->keys.as<uint64_t>(),
                                                         b->perm.as<int32_t>());
    else
        k_seg_morton<2><<<grid_for(n, 256), 256, 0, s>>>(b->pos.as<double>(), n,
                                                         b->sys_of.as<int32_t>(),
                                                         b->box.as<double>(),
                                                         b->keys.as<uint64_t>(),
                                                         b->perm.as<int32_t>());
    BHUT_CUDA(cudaGetLastError());
    note_launches(4);
    BHUT_TRY(radix_sort_pairs(b->keys.as<uint64_t>(), b->perm.as<int32_t>(), n,
                              dim == 3 ? 63 : 42, b->sort_scratch.p, s));
    if (ns > 1) {
        k_seg_key2<<<grid_for(n, 256), 256, 0, s>>>(b->perm.as<int32_t>(), b->sys_of.as<int32_t>(),
                                                     n, b->key2.as<uint64_t>());
        BHUT_CUDA(cudaGetLastError());
        note_launches(1);
        BHUT_TRY(radix_sort_pairs(b->key2.as<uint64_t>(), b->perm.as<int32_t>(), n,
                                  bits_for(ns - 1), b->sort_scratch.p, s));
    }
    if (b->keep_active) {
        if (b->refit_rule) {
            k_seg_keep_outside<<<grid_for(n, 256), 256, 0, s>>>(
                b->pos.as<double>(), n, dim, b->sys_of.as<int32_t>(), b->roots.as<double>(),
                b->keep.as<uint8_t>(), b->acc.as<uint64_t>());
            k_seg_keep_finish<<<gs, 128, 0, s>>>(b->acc.as<uint64_t>(), ns,
                                                  b->keep.as<uint8_t>(), b->forced.as<int32_t>());
            BHUT_CUDA(cudaGetLastError());
            note_launches(2);
        }
        k_seg_keep_perm<<<grid_for(n, 256), 256, 0, s>>>(n, b->sys_of.as<int32_t>(),
                                                          b->keep.as<uint8_t>(),
                                                          b->perm_in.as<int32_t>(),
                                                          b->perm.as<int32_t>());
        BHUT_CUDA(cudaGetLastError());
        note_launches(1);
    }
    BHUT_TRY(launch_gather(b->pos.as<double>(), b->mass.as<double>(), b->perm.as<int32_t>(), n,
                           dim, b->sx.as<double>(), b->sy.as<double>(), b->sz.as<double>(),
                           b->sm.as<double>(), s));
    NodeOut o{b->cm.as<NodeCM>(), b->size.as<double>(), b->center.as<double>(),
              b->half.as<double>(), b->lo.as<double>(), b->hi.as<double>()};
    BHUT_TRY(launch_bottom_up(b->dev(), b->leaf_list.as<int32_t>(), b->ltot,
                              b->first_child.as<int32_t>(), b->start.as<int32_t>(),
                              b->count.as<int32_t>(), b->parent.as<int32_t>(),
                              b->arrive.as<unsigned>(), o, false, nullptr, nullptr,
                              b->frontier.as<int32_t>(), b->counter.as<unsigned>() + 2,
                              b->err.as<unsigned>(), s));
    if (b->refit_rule) {
        k_seg_roots_update<<<grid_for(ns, 128), 128, 0, s>>>(
            b->d_node_off.as<int64_t>(), b->center.as<double>(), b->half.as<double>(), dim, ns,
            b->keep_active ? b->keep.as<uint8_t>() : nullptr, b->roots.as<double>());
        BHUT_CUDA(cudaGetLastError());
        note_launches(1);
    }
    const bool quad = b->form == BHUT_FORM_FP32 && b->multipole == BHUT_MULTIPOLE_QUAD;
    if (quad)
        BHUT_TRY(launch_quadrupoles(b->dev(), b->leaf_list.as<int32_t>(), b->ltot,
                                    b->first_child.as<int32_t>(), b->start.as<int32_t>(),
                                    b->count.as<int32_t>(), b->parent.as<int32_t>(),
                                    b->arrive.as<unsigned>(), b->quad.as<double>(),
                                    b->frontier.as<int32_t>(), b->counter.as<unsigned>() + 2,
                                    b->err.as<unsigned>(), s));
    k_seg_ff_particles<<<grid_for(n, 256), 256, 0, s>>>(b->dev(), b->sys_of.as<int32_t>(),
                                                        b->frames.as<FastFrame>(),
                                                        b->ph.as<float4>(), b->pl.as<float4>());
    k_seg_ff_nodes<<<grid_for(b->mtot, 256), 256, 0, s>>>(
        b->dev(), b->node_sys.as<int32_t>(), b->frames.as<FastFrame>(), b->center.as<double>(),
        b->nh.as<float4>(), b->nl.as<float4>(), b->nsize.as<float>(), b->ndelta.as<float>(),
        quad ? b->quad.as<double>() : nullptr, b->nq0.as<float4>(), b->nq1.as<float2>(),
        b->nhdr.as<int4>());
    BHUT_CUDA(cudaGetLastError());
    note_launches(2);
    // traversal
    BHUT_CUDA(cudaMemsetAsync(b->counter.p, 0, sizeof(unsigned), s));
    BHUT_CUDA(cudaMemsetAsync(b->stats.p, 0, sizeof(unsigned long long) * 8, s));
    BatchDev bd{b->dev(), b->d_part_off.as<int64_t>(), b->d_node_off.as<int64_t>(),
                b->frames.as<FastFrame>(), b->ph.as<float4>(), b->pl.as<float4>(),
                b->nh.as<float4>(), b->nl.as<float4>(), b->nsize.as<float>(),
                b->ndelta.as<float>(), quad ? b->nq0.as<float4>() : nullptr,
                quad ? b->nq1.as<float2>() : nullptr, b->nhdr.as<int4>()};
    BatchArgs a{b->d_tasks.as<int2>(), (int)b->tasks.size(), b->counter.as<unsigned>(), theta,
                eps, G, b->mac, out, b->err.as<unsigned>(), b->stats.as<unsigned long long>()};
    const bool fp32 = b->form == BHUT_FORM_FP32;
    const int stk = b->stack;
    if (b->ev_trav[0]) BHUT_TRY(record_timing_event(b->ev_trav[0], s));
    if (dim == 3) {
        if (fp32 && b->tpw == 32) launch_batch_traverse<3, true, 32>(stk, s, bd, a);
        else if (fp32) launch_batch_traverse<3, true, 16>(stk, s, bd, a);
        else if (b->tpw == 32) launch_batch_traverse<3, false, 32>(stk, s, bd, a);
        else launch_batch_traverse<3, false, 16>(stk, s, bd, a);
    } else {
        if (fp32) launch_batch_traverse<2, true, 32>(stk, s, bd, a);
        else launch_batch_traverse<2, false, 32>(stk, s, bd, a);
    }
    BHUT_CUDA(cudaGetLastError());
    if (b->ev_trav[1]) BHUT_TRY(record_timing_event(b->ev_trav[1], s));
    note_launches(1);
    return kOk;
}

int ensure_topology(bhut_batch* b)
{
    if (b->topo_valid) return kOk;
    k_seg_topology<<<(unsigned)b->nsys, kSegThreads, 0, b->stream>>>(
        b->d_part_off.as<int64_t>(), b->d_node_off.as<int64_t>(), b->d_leaf_off.as<int64_t>(),
        b->leaf, b->first_child.as<int32_t>(), b->start.as<int32_t>(), b->count.as<int32_t>(),
        b->parent.as<int32_t>(), b->leaf_list.as<int32_t>(), b->err.as<unsigned>());
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    // leaves in particle order (the particle keys are free until the solve)
    BHUT_TRY(order_leaves(b->leaf_list.as<int32_t>(), b->ltot, b->start.as<int32_t>(),
                          b->keys.as<uint64_t>(), b->sort_scratch.p, b->stream));
    b->topo_valid = true;
    return kOk;
}

int check_batch_err(bhut_batch* b)
{
    unsigned e = 0;
    BHUT_CUDA(cudaMemcpyAsync(&e, b->err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, b->stream));
    BHUT_CUDA(cudaMemcpyAsync(b->last_stats, b->stats.p, sizeof(unsigned long long) * 5,
                              cudaMemcpyDeviceToHost, b->stream));
    BHUT_CUDA(cudaStreamSynchronize(b->stream));
    if (!e) return kOk;
    BHUT_CUDA(cudaMemsetAsync(b->err.p, 0, sizeof(unsigned), b->stream));
    if (e & kErrNonFinite) { set_error("positions and masses must be finite"); return kInvalid; }
    set_error("device error word 0x%x in batched solve", e);
    return kDeviceFlag;
}

}  // namespace

extern "C" {

int bhut_batch_create(int dim, int leaf_size, void* stream, bhut_batch** out)
{
    if (!out) { set_error("out is NULL"); return kInvalid; }
    *out = nullptr;
    if (dim != 2 && dim != 3) { set_error("dim must be 2 or 3, got %d", dim); return kInvalid; }
    if (leaf_size <= 0) { set_error("leaf_size must be positive, got %d", leaf_size); return kInvalid; }
    bhut_batch* b = new bhut_batch();
    b->dim = dim;
    b->leaf = leaf_size;
    if (stream) {
        b->stream = (cudaStream_t)stream;
    } else {
        cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) { delete b; return cuda_status(e, "cudaStreamCreate"); }
        b->own_stream = true;
    }
    for (cudaEvent_t& e : b->ev_trav)
        if (cudaEventCreate(&e) != cudaSuccess) { cudaGetLastError(); e = nullptr; }
    *out = b;
    return kOk;
}

int bhut_batch_configure(bhut_batch* b, int form, int criterion, int targets_per_warp,
                         int use_graph)
{
    if (!b) { set_error("batch is NULL"); return kInvalid; }
    if (form != BHUT_FORM_FAST && form != BHUT_FORM_FP32) {
        set_error("the batched solver runs form fast or fp32, got %d", form);
        return kInvalid;
    }
    if (criterion != BHUT_MAC_BH && criterion != BHUT_MAC_OFFSET) {
        set_error("unknown opening criterion %d", criterion);
        return kInvalid;
    }
    if (criterion == BHUT_MAC_OFFSET && form != BHUT_FORM_FP32) {
        set_error("the offset criterion is available with the fp32 form only");
        return kInvalid;
    }
    if (targets_per_warp != 32 && targets_per_warp != 16) {
        set_error("targets_per_warp must be 32 or 16, got %d", targets_per_warp);
        return kInvalid;
    }
    if (targets_per_warp == 16 && b->dim != 3) {
        set_error("targets_per_warp = 16 is built for dim = 3 only");
        return kInvalid;
    }
    const bool retask = targets_per_warp != b->tpw;
    b->form = form;
    b->mac = criterion;
    b->tpw = targets_per_warp;
    b->use_graph = use_graph != 0;
    drop_graph(b);
    if (retask && b->layout_valid) BHUT_TRY(plan_tasks(b));
    return kOk;
}

int bhut_batch_set_multipole(bhut_batch* b, int multipole)
{
    if (!b) { set_error("batch is NULL"); return kInvalid; }
    if (multipole != BHUT_MULTIPOLE_MONO && multipole != BHUT_MULTIPOLE_QUAD) {
        set_error("unknown multipole order %d", multipole);
        return kInvalid;
    }
    if (multipole != b->multipole) drop_graph(b);
    b->multipole = multipole;
    return kOk;
}

int bhut_batch_set_stack(bhut_batch* b, int placement)
{
    if (!b) { set_error("batch is NULL"); return kInvalid; }
    if (placement != BHUT_STACK_SHARED && placement != BHUT_STACK_REGISTERS) {
        set_error("unknown stack placement %d", placement);
        return kInvalid;
    }
    if (placement != b->stack) drop_graph(b);
    b->stack = placement;
    return kOk;
}

int bhut_batch_load(bhut_batch* b, const double* positions, const double* masses,
                    const int64_t* offsets, int64_t nsys)
{
    if (!b) { set_error("batch is NULL"); return kInvalid; }
    if (nsys <= 0 || !offsets || !positions || !masses) { set_error("empty batch"); return kInvalid; }
    if (offsets[0] != 0) { set_error("offsets[0] must be 0"); return kInvalid; }
    bool same = b->layout_valid && b->nsys == nsys &&
                std::memcmp(b->part_off.data(), offsets, sizeof(int64_t) * (nsys + 1)) == 0;
    if (!same) BHUT_TRY(plan_layout(b, offsets, nsys));
    cudaStream_t s = b->stream;
    BHUT_CUDA(cudaMemcpyAsync(b->pos.p, positions, sizeof(double) * b->ntot * b->dim,
                              is_device_pointer(positions) ? cudaMemcpyDeviceToDevice
                                                           : cudaMemcpyHostToDevice, s));
    BHUT_CUDA(cudaMemcpyAsync(b->mass.p, masses, sizeof(double) * b->ntot,
                              is_device_pointer(masses) ? cudaMemcpyDeviceToDevice
                                                        : cudaMemcpyHostToDevice, s));
    b->built = true;
    return kOk;
}

int bhut_batch_solve(bhut_batch* b, double theta, double softening, double G, double* out)
{
    if (!b) { set_error("batch is NULL"); return kInvalid; }
    if (!b->built) { set_error("load systems before solving"); return kNotBuilt; }
    if (!(theta >= 0)) { set_error("theta must be non-negative, got %g", theta); return kInvalid; }
    if (!(softening >= 0)) { set_error("softening must be non-negative, got %g", softening); return kInvalid; }
    BHUT_TRY(ensure_topology(b));
    const bool dev_out = is_device_pointer(out);
    double* dst = dev_out ? out : b->out.as<double>();
    {
        const bool fp32 = b->form == BHUT_FORM_FP32;
        if (b->dim == 3) {
            if (fp32 && b->tpw == 32) prime_grid_of<3, true, 32>(b->stack);
            else if (fp32) prime_grid_of<3, true, 16>(b->stack);
            else if (b->tpw == 32) prime_grid_of<3, false, 32>(b->stack);
            else prime_grid_of<3, false, 16>(b->stack);
        } else {
            if (fp32) prime_grid_of<2, true, 32>(b->stack);
            else prime_grid_of<2, false, 32>(b->stack);
        }
    }
    if (b->use_graph) {
        if (!b->graph || theta != b->g_theta || softening != b->g_eps || G != b->g_G ||
            dst != b->g_out) {
            drop_graph(b);
            cudaGraph_t g;
            BHUT_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
            int st = enqueue_solve(b, theta, softening, G, dst);
            cudaError_t e = cudaStreamEndCapture(b->stream, &g);
            if (st != kOk) { if (e == cudaSuccess) cudaGraphDestroy(g); return st; }
            BHUT_CUDA(e);
            e = cudaGraphInstantiate(&b->graph, g, 0);
            cudaGraphDestroy(g);
            BHUT_CUDA(e);
            b->g_theta = theta; b->g_eps = softening; b->g_G = G; b->g_out = dst;
        }
        BHUT_CUDA(cudaGraphLaunch(b->graph, b->stream));
    } else {
        BHUT_TRY(enqueue_solve(b, theta, softening, G, dst));
    }
    if (!dev_out)
        BHUT_CUDA(cudaMemcpyAsync(out, dst, sizeof(double) * b->ntot * b->dim,
                                  cudaMemcpyDeviceToHost, b->stream));
    return check_batch_err(b);
}

int bhut_batch_keep_order(bhut_batch* b, const uint8_t* keep, const int32_t* perm)
{
    if (!b) { set_error("batch is NULL"); return kInvalid; }
    if (!b->layout_valid) { set_error("load systems first"); return kNotBuilt; }
    cudaStream_t s = b->stream;
    if (!keep) {
        if (b->keep_active) drop_graph(b);
        b->keep_active = false;
        return kOk;
    }
    if (!perm) { set_error("perm is NULL"); return kInvalid; }
    BHUT_CUDA(cudaMemcpyAsync(b->keep.p, keep, b->nsys, is_device_pointer(keep)
                              ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
    BHUT_CUDA(cudaMemcpyAsync(b->perm_in.p, perm, sizeof(int32_t) * b->ntot,
                              is_device_pointer(perm) ? cudaMemcpyDeviceToDevice
                                                      : cudaMemcpyHostToDevice, s));
    if (!b->keep_active) drop_graph(b);
    b->keep_active = true;
    return kOk;
}

int bhut_batch_set_refit_rule(bhut_batch* b, int on)
{
    if (!b) { set_error("batch is NULL"); return kInvalid; }
    if ((on != 0) != b->refit_rule) drop_graph(b);
    b->refit_rule = on != 0;
    return kOk;
}

int bhut_batch_set_roots(bhut_batch* b, const double* roots)
{
    if (!b) { set_error("batch is NULL"); return kInvalid; }
    if (!b->layout_valid || !roots) { set_error("load systems first"); return kInvalid; }
    BHUT_CUDA(cudaMemcpyAsync(b->roots.p, roots, sizeof(double) * 4 * b->nsys, cudaMemcpyDefault,
                              b->stream));
    if (!is_device_pointer(roots)) BHUT_CUDA(cudaStreamSynchronize(b->stream));
    return kOk;
}

int bhut_batch_forced(const bhut_batch* b, int32_t* counts)
{
    if (!b) { set_error("batch is NULL"); return kInvalid; }
    if (!b->layout_valid || !counts) { set_error("nothing to copy"); return kInvalid; }
    BHUT_CUDA(cudaMemcpyAsync(counts, b->forced.p, sizeof(int32_t) * b->nsys, cudaMemcpyDefault,
                              b->stream));
    BHUT_CUDA(cudaStreamSynchronize(b->stream));
    return kOk;
}

int bhut_batch_roots(const bhut_batch* b, double* roots)
{
    if (!b) { set_error("batch is NULL"); return kInvalid; }
    if (!b->layout_valid || !roots) { set_error("nothing to copy"); return kInvalid; }
    cudaStream_t s = b->stream;
    if (b->refit_rule) {   // the roots kept by the solves
        BHUT_CUDA(cudaMemcpyAsync(roots, b->roots.p, sizeof(double) * 4 * b->nsys,
                                  cudaMemcpyDefault, s));
        BHUT_CUDA(cudaStreamSynchronize(s));
        return kOk;
    }
    BufB tmp;
    BHUT_TRY(tmp.ensure(sizeof(double) * 4 * b->nsys, s));
    k_seg_roots<<<grid_for(b->nsys, 128), 128, 0, s>>>(b->d_node_off.as<int64_t>(),
                                                        b->center.as<double>(),
                                                        b->half.as<double>(), b->dim, b->nsys,
                                                        tmp.as<double>());
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    BHUT_CUDA(cudaMemcpyAsync(roots, tmp.p, sizeof(double) * 4 * b->nsys, cudaMemcpyDefault, s));
    BHUT_CUDA(cudaStreamSynchronize(s));
    tmp.release(s);
    return kOk;
}

int bhut_batch_outside(const bhut_batch* b, const double* roots, uint8_t* flags)
{
    if (!b) { set_error("batch is NULL"); return kInvalid; }
    if (!b->layout_valid || !roots || !flags) { set_error("load systems first"); return kInvalid; }
    cudaStream_t s = b->stream;
    BufB droots, dflags;
    BHUT_TRY(droots.ensure(sizeof(double) * 4 * b->nsys, s));
    BHUT_TRY(dflags.ensure(b->nsys, s));
    BHUT_CUDA(cudaMemcpyAsync(droots.p, roots, sizeof(double) * 4 * b->nsys, cudaMemcpyDefault, s));
    k_seg_outside<<<(unsigned)b->nsys, kSegThreads, 0, s>>>(b->pos.as<double>(),
                                                           b->d_part_off.as<int64_t>(),
                                                           droots.as<double>(), b->dim,
                                                           dflags.as<uint8_t>());
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    BHUT_CUDA(cudaMemcpyAsync(flags, dflags.p, b->nsys, cudaMemcpyDefault, s));
    BHUT_CUDA(cudaStreamSynchronize(s));
    droots.release(s);
    dflags.release(s);
    return kOk;
}

int bhut_batch_order(const bhut_batch* b, int32_t* perm)
{
    if (!b) { set_error("batch is NULL"); return kInvalid; }
    if (!b->layout_valid || !perm) { set_error("nothing to copy"); return kInvalid; }
    BHUT_CUDA(cudaMemcpyAsync(perm, b->perm.p, sizeof(int32_t) * b->ntot, cudaMemcpyDefault,
                              b->stream));
    if (!is_device_pointer(perm)) BHUT_CUDA(cudaStreamSynchronize(b->stream));
    return kOk;
}

int bhut_leapfrog(double* positions, double* velocities, const double* accelerations, int64_t n,
                  int dim, double kick, double drift, void* stream)
{
    if (n <= 0) return kOk;
    if (dim != 2 && dim != 3) { set_error("dim must be 2 or 3, got %d", dim); return kInvalid; }
    if (!is_device_pointer(positions) || !is_device_pointer(velocities) ||
        !is_device_pointer(accelerations)) {
        set_error("bhut_leapfrog needs device pointers");
        return kInvalid;
    }
    const int64_t m = n * dim;
    k_leapfrog<<<grid_for(m, 256), 256, 0, (cudaStream_t)stream>>>(positions, velocities,
                                                                   accelerations, m, kick, drift);
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    return kOk;
}

int bhut_batch_info(const bhut_batch* b, int64_t* nsys, int64_t* n_total, int64_t* nodes_total,
                    int64_t* tasks)
{
    if (!b) { set_error("batch is NULL"); return kInvalid; }
    if (nsys) *nsys = b->nsys;
    if (n_total) *n_total = b->ntot;
    if (nodes_total) *nodes_total = b->mtot;
    if (tasks) *tasks = (int64_t)b->tasks.size();
    return kOk;
}

int bhut_batch_stats(const bhut_batch* b, int64_t* p2p, int64_t* m2p, int64_t* visits)
{
    if (!b) { set_error("batch is NULL"); return kInvalid; }
    if (p2p) *p2p = (int64_t)b->last_stats[0];
    if (m2p) *m2p = (int64_t)b->last_stats[1];
    if (visits) *visits = (int64_t)b->last_stats[2];
    return kOk;
}

void bhut_batch_destroy(bhut_batch* b)
{
    if (!b) return;
    drop_graph(b);
    b->release_all();
    cudaStreamSynchronize(b->stream);
    for (cudaEvent_t e : b->ev_trav)
        if (e) cudaEventDestroy(e);
    if (b->own_stream) cudaStreamDestroy(b->stream);
    delete b;
}

int bhut_batch_traverse_ms(const bhut_batch* b, double* ms)
{
    if (!b || !ms) { set_error("batch or ms is NULL"); return kInvalid; }
    if (!b->ev_trav[0] || !b->ev_trav[1]) { set_error("no traversal timing events"); return kInvalid; }
    BHUT_CUDA(cudaEventSynchronize(b->ev_trav[1]));
    float f = 0.0f;
    BHUT_CUDA(cudaEventElapsedTime(&f, b->ev_trav[0], b->ev_trav[1]));
    *ms = f;
    return kOk;
}

}  // extern "C"
