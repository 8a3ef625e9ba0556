// Device-side tree layout shared by the build, refit and traversal kernels.
#pragma once
#include "common.cuh"

namespace bhut {

// Centre of mass and mass of a node, one 32-byte load.
struct __align__(32) NodeCM {
    double x, y, z, w;
};

// Node arrays are indexed by the reference's node id (bhut/tree/build.py:
// the k-th internal node in pop order of the build stack has children 2k+1
// and 2k+2).  Particles are held as Morton-sorted SoA.
struct TreeDev {
    int dim;
    int leaf_size;
    int64_t n;              // particles
    int64_t m;              // nodes
    // Morton-sorted particles (SoA) and their original indices
    const double* sx;
    const double* sy;
    const double* sz;
    const double* sm;
    const int32_t* perm;
    // nodes
    const NodeCM* cm;      // (com.x, com.y, com.z, mass)
    const double* size;     // 2 * half_size (the opening-test node size)
    const int32_t* first_child;  // -1 for a leaf
    const int32_t* start;
    const int32_t* count;
};

// Geometry of the count-split topology for (n, leaf_size).  The counts at
// depth d are floor(n / 2^d) or that plus one, so per depth only two count
// values and two subtree internal-node counts exist.
constexpr int kMaxDepth = 64;
constexpr int kMaxClimb = 2 * kMaxDepth;   // bound of every leaf-to-root climb
struct TopoTables {
    int depth;                     // deepest level (all nodes there are leaves)
    int64_t n;
    int leaf_size;
    int64_t cnt_lo[kMaxDepth];     // floor(n / 2^d)
    int64_t internal[kMaxDepth][2];  // internal-node count of a subtree with cnt_lo[d] + {0,1}
    int64_t num_nodes;
    int64_t num_leaves;
    int64_t slots;                 // 2^(depth+1) - 1 BFS slots
};

int make_topo_tables(int64_t n, int leaf_size, TopoTables* t);

// Normalisation of the "fast" traversal: u = (x - c) * s with s a power of
// two mapping the box into [-1, 1]; masses scaled by ms (a power of two, or
// 1 / m0 when every particle has the same mass m0: unit = 1, particle masses
// exactly 1); physical acceleration = normalised acceleration * conv
// (= s^2 / ms, or s^2 m0).
struct FastFrame {
    double c[3];
    double s;
    double ms;
    double conv;
    int unit;
};

// Float-float copies of the particles (Morton order) and nodes.
struct FastTree {
    const FastFrame* frame;
    const float4* ph;   // (x, y, z, m) hi
    const float4* pl;   // (x, y, z, m) lo
    const float4* nh;   // (com, mass) hi per node
    const float4* nl;   // (com, mass) lo per node
    const float* nsize; // 2 * half_size, normalised, per node
    const float* ndelta; // |com - AABB centre|, normalised, per node (offset criterion)
    const float4* nq0;   // quadrupole (xx, yy, zz, xy), normalised, per node; NULL: monopoles
    const float2* nq1;   // quadrupole (xz, yz)
    const int4* nhdr;    // per node, one load per visit: leaf (-1, start, count, mass != 0),
                         // internal (first child, size, |com - centre| as float bits, mass != 0)
};

// Morton encoding (bhut/utils/morton.py:14-45, 183-198) and the quantisation
// of bhut/space/bbox.py:85-94, shared by the single-tree and batched builds.
static __device__ __forceinline__ uint64_t expand3(uint64_t x)
{
    x = (x | (x << 32)) & 0x1F00000000FFFFull;
    x = (x | (x << 16)) & 0x1F0000FF0000FFull;
    x = (x | (x << 8)) & 0x100F00F00F00F00Full;
    x = (x | (x << 4)) & 0x10C30C30C30C30C3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

static __device__ __forceinline__ uint64_t expand2(uint64_t x)
{
    x = (x | (x << 16)) & 0x0000FFFF0000FFFFull;
    x = (x | (x << 8)) & 0x00FF00FF00FF00FFull;
    x = (x | (x << 4)) & 0x0F0F0F0F0F0F0F0Full;
    x = (x | (x << 2)) & 0x3333333333333333ull;
    x = (x | (x << 1)) & 0x5555555555555555ull;
    return x;
}

// p01 = (x - pmin) / extent + offset, clamped at 1 - 1e-12 (bbox.py:85-94);
// coordinate = trunc(p01 * 2^21) clamped to 2^21 - 1 (morton.py:183-185).
static __device__ __forceinline__ uint64_t quantise(double x, double pmin, double extent, double offset)
{
    const double top = 1.0 - 1e-12;
    double p = __dadd_rn(__ddiv_rn(__dsub_rn(x, pmin), extent), offset);
    p = p > top ? top : p;
    uint64_t q = __double2ull_rz(__dmul_rn(p, 2097152.0));
    return q < 2097151ull ? q : 2097151ull;
}

// The same quantised coordinate with two FP64 operations instead of a
// division: with y = RN(1/extent), q0 = RN(RN(x - pmin) * y) lies within
// 3 * 2^-53 of RN(RN(x - pmin) / extent) (both are within that of the exact
// quotient, which is at most 1), i.e. within 3 * 2^-32 in units of the
// 2^-21 grid.  When q0 * 2^21 is at least 2^-29 away from every integer its
// truncation is the reference's; otherwise (an exact grid point, a tiny
// quotient: a few coordinates per build) the division is taken after all.
// q0 * 2^21 is read from the bits of q0 (a power-of-two scaling is exact).
// Only for offset == 0 (offset 0.5 marks a degenerate axis: exact path).
static __device__ __forceinline__ uint64_t quantise_rcp(double x, double pmin, double extent,
                                                        double rcp)
{
    const double a = __dsub_rn(x, pmin);
    const uint64_t b = (uint64_t)__double_as_longlong(__dmul_rn(a, rcp));
    if (b == 0) return 0;                            // a == 0: quotient exactly 0
    const int e = (int)((b >> 52) & 0x7ff);
    const uint64_t m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int s = 1054 - e;                          // fractional bits of q0 * 2^21
    uint64_t k;
    bool ok;
    if ((b >> 63) || e == 0 || s < 1 || s > 80) {
        k = 0;
        ok = false;
    } else if (s <= 52) {
        k = m >> s;
        const uint64_t frac = m & ((1ull << s) - 1);
        const uint64_t thr = s > 29 ? (1ull << (s - 29)) : 1ull;
        ok = frac >= thr && ((1ull << s) - frac) >= thr;
    } else {                                         // q0 * 2^21 < 1
        k = 0;
        ok = s > 53 || m <= (1ull << 53) - (1ull << 25);
    }
    if (!ok) return quantise(x, pmin, extent, 0.0);
    return k < 2097151ull ? k : 2097151ull;
}

// Order-preserving integer images of doubles (min/max on the integer pipe,
// and with 64-bit integer atomics): ord_key(a) < ord_key(b) iff a < b for
// non-NaN a, b (-0 before +0).
static __device__ __forceinline__ uint64_t ord_key(uint64_t b)
{
    return b ^ ((uint64_t)((int64_t)b >> 63) | 0x8000000000000000ull);
}
static __device__ __forceinline__ uint64_t ord_inv(uint64_t k)
{
    return k ^ (((k >> 63) ? 0ull : ~0ull) | 0x8000000000000000ull);
}
static __device__ __forceinline__ bool finite_bits(uint64_t b)
{
    return ((b >> 52) & 0x7ff) != 0x7ff;
}

static __device__ __forceinline__ uint64_t morton3(uint64_t cx, uint64_t cy, uint64_t cz)
{
    return expand3(cx) | (expand3(cy) << 1) | (expand3(cz) << 2);
}

static __device__ __forceinline__ uint64_t morton2(uint64_t cx, uint64_t cy)
{
    return expand2(cx) | (expand2(cy) << 1);
}

// Node arrays written by the bottom-up pass.
struct NodeOut {
    NodeCM* cm;        // (com, mass)
    double* size;       // 2 * half_size
    double* center;     // dim per node
    double* half;
    double* lo;         // 3 per node (AABB scratch)
    double* hi;
};

// Kernel launchers (build.cu, traverse.cu).
// Bounding box: box[0..2] = min, box[3..5] = max, box[6] = max |mass| (0
// without masses), box[8..10] = RN(1 / (max - min)) per axis (1 for a zero
// extent), box[11] = 1 if an axis has zero extent, box[12..14] = 1 if the
// axis holds a NaN, box[15] = 1 if every mass equals mass[0] > 0 (finite).
// `partial` holds kBoxPartialDoubles doubles.
constexpr unsigned kBoxMaxBlocks = 152u * 4u;
constexpr int kBoxPartialDoubles = 8 * (int)kBoxMaxBlocks;
constexpr int kBoxDoubles = 16;
int launch_bbox(const double* pos, const double* mass, int64_t n, int dim, double* partial,
                unsigned* counter, double* box, unsigned* err, cudaStream_t s);
// The same box while copying positions and masses to pos_copy / mass_copy
// (either may be NULL); a non-finite value sets kErrNonFinite in *err.
int launch_stage_bbox(const double* pos, const double* mass, int64_t n, int dim, double* pos_copy,
                      double* mass_copy, double* partial, unsigned* counter, double* box,
                      unsigned* err, cudaStream_t s);
int launch_morton(const double* pos, int64_t n, int dim, const double* box, uint64_t* keys,
                  int32_t* idx, cudaStream_t s);
int launch_gather(const double* pos, const double* mass, const int32_t* perm, int64_t n, int dim,
                  double* sx, double* sy, double* sz, double* sm, cudaStream_t s);
int launch_topology(const TopoTables& tt, int32_t* first_child, int32_t* start, int32_t* count,
                    int32_t* parent, int32_t* leaf_list, unsigned* leaf_counter, unsigned* err,
                    cudaStream_t s);
// Reorders the leaf list by first particle (siblings end up in neighbouring
// entries, which the bottom-up pass merges inside a block).  `keys` holds
// num_leaves entries; the scratch sort_scratch_bytes(num_leaves).
int order_leaves(int32_t* leaf_list, int64_t num_leaves, const int32_t* start, uint64_t* keys,
                 void* sort_scratch, cudaStream_t s);
// Node boxes and moments from the leaves up (build, or refit with opos /
// omass in input order); quadrupoles the same way.  `frontier` holds
// num_leaves entries of scratch, `frontier_count` one counter.
int launch_bottom_up(const TreeDev& t, const int32_t* leaf_list, int64_t num_leaves,
                     const int32_t* first_child, const int32_t* start, const int32_t* count,
                     const int32_t* parent, unsigned* arrive, NodeOut o, bool refit,
                     const double* opos, const double* omass, int32_t* frontier,
                     unsigned* frontier_count, unsigned* err, cudaStream_t s);
int launch_quadrupoles(const TreeDev& t, const int32_t* leaf_list, int64_t num_leaves,
                       const int32_t* first_child, const int32_t* start, const int32_t* count,
                       const int32_t* parent, unsigned* arrive, double* quad, int32_t* frontier,
                       unsigned* frontier_count, unsigned* err, cudaStream_t s);
int launch_outside_root(const double* pos, int64_t n, int dim, const double* center0,
                        const double* half0, unsigned* flag, cudaStream_t s);
int launch_traverse_exact(const TreeDev& t, const double* tx, const double* ty, const double* tz,
                          const int32_t* self_id, const int32_t* out_idx, int64_t nt, double theta,
                          double eps, double G, double* out, unsigned* err,
                          unsigned long long* stats, cudaStream_t s);
int launch_fast_prepare(const double* box, int dim, FastFrame* frame, const TreeDev& t,
                        const double* center, float4* ph, float4* pl, float4* nh, float4* nl,
                        float* nsize, float* ndelta, const double* quad, float4* nq0,
                        float2* nq1, int4* nhdr, cudaStream_t s);
int launch_fast_targets(const double* tx, const double* ty, const double* tz, int64_t nt, int dim,
                        const FastFrame* frame, float4* th, float4* tl, cudaStream_t s);
int launch_traverse_fast(const TreeDev& t, const FastTree& ft, const float4* th, const float4* tl,
                         const double* tx, const double* ty, const double* tz,
                         const int32_t* self_id, const int32_t* out_idx, int64_t nt, double theta,
                         double eps, double G, double eps_scaled_sq, double* out, unsigned* err,
                         unsigned long long* stats, cudaStream_t s, bool fp32, int mac);
// TreeData arrays as the reference lays them out (bhut/tree/node.py:15-77):
// int64 indices, com (m, dim), for compute_tree_statistics.
struct StatTree {
    const double* com;
    const double* half_size;
    const double* mass;
    const int64_t* first_child;
    const int64_t* child_count;
    const int64_t* start;
    const int64_t* count;
    int64_t m;
};
int launch_tree_statistics(const StatTree& t, int dim, const double* targets, int64_t nt,
                           double theta, unsigned long long* totals, unsigned* err,
                           cudaStream_t s);

// stages.cu
int launch_normalize(const double* pts, int64_t n, int dim, const double* pmin, const double* pmax,
                     double top, double* out, cudaStream_t s);
int launch_morton_unit(const double* p01, int64_t n, int dim, int bits, uint64_t* codes,
                       unsigned* bad, cudaStream_t s);
int launch_gather_rows(const void* src, int64_t n, int64_t row_bytes, const int64_t* perm,
                       void* dst, unsigned* err, cudaStream_t s);
int launch_import_nodes(const int64_t* fc, const int64_t* cc, const int64_t* st, const int64_t* ct,
                        const double* half_in, const double* mass_in, const double* com_in,
                        const double* center_in, int64_t m, int64_t n, int dim,
                        int32_t* first_child, int32_t* start, int32_t* count, int32_t* parent,
                        NodeCM* cm, double* size, double* half, double* center,
                        int32_t* leaf_list, unsigned* leaf_counter, unsigned* err, cudaStream_t s);
int launch_import_perm(const int64_t* in, int64_t n, int32_t* out, unsigned* err, cudaStream_t s);
int launch_iota(int32_t* out, int64_t n, cudaStream_t s);
int launch_widen_i32(const int32_t* in, int64_t n, int64_t* out, cudaStream_t s);
int measure_fp32_peak(double* tflops);

int direct_chunks(int64_t n, int64_t nt);
int launch_direct(const double* pos, const double* mass, int64_t n, int dim, const double* targets,
                  const int64_t* self_id, int64_t nt, double eps, double G, double* out,
                  double* partial, int chunks, cudaStream_t s);

}  // namespace bhut
