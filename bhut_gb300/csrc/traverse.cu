// Barnes-Hut traversal, FP64 "exact" form, and the FP64 direct-sum kernel.
//
// k_traverse_exact replaces the per-target loop of bhut/traverse/bh.py:
// _barnes_hut_single_target (:485-548, self) and
// _barnes_hut_single_target_external (:83-146).  One warp owns 32
// Morton-contiguous targets and walks the tree with a shared stack of
// (node, lane mask) entries: a lane that accepts a node adds its monopole and
// drops out of that subtree, so every lane visits exactly the nodes, in
// exactly the order, of the reference's own traversal for its target
// (right child first, bh.py:531-537).  Per-pair arithmetic is the Numba leaf
// loop (bh.py:226-280) with explicit round-to-nearest intrinsics and IEEE
// sqrt/division, so P2P terms match the reference's bit for bit; monopoles
// use r2^1.5 = r2 * sqrt(r2) in place of pow (kernels.py:66), within 2 ulp.
#include "tree.cuh"

namespace bhut {

constexpr int kTravWarps = 4;
constexpr int kTravThreads = kTravWarps * kWarp;

// bh.py:576-601 with np.linalg.norm = sqrt(fma chain) (OpenBLAS ddot).
template <int DIM>
__device__ __forceinline__ bool open_exact(double x, double y, double z, NodeCM cm, double size,
                                           double theta)
{
    double dx = __dsub_rn(x, cm.x), dy = __dsub_rn(y, cm.y);
    double s;
    if (DIM == 3) {
        double dz = __dsub_rn(z, cm.z);
        s = __fma_rn(dz, dz, __fma_rn(dy, dy, __dmul_rn(dx, dx)));
    } else {
        s = __fma_rn(dy, dy, __dmul_rn(dx, dx));
    }
    double d = __dsqrt_rn(s);
    if (d == 0.0) return true;
    return __ddiv_rn(size, d) >= theta;
}

// kernels.py:52-69 acc_monopole (single vector) via acc_monopole_node.
template <int DIM>
__device__ __forceinline__ void monopole_exact(double x, double y, double z, NodeCM cm,
                                               double eps2, double G, double& ax, double& ay,
                                               double& az)
{
    double dx = __dsub_rn(cm.x, x), dy = __dsub_rn(cm.y, y);
    double dz = DIM == 3 ? __dsub_rn(cm.z, z) : 0.0;
    double r2 = __dadd_rn(__dadd_rn(-0.0, __dmul_rn(dx, dx)), __dmul_rn(dy, dy));
    if (DIM == 3) r2 = __dadd_rn(r2, __dmul_rn(dz, dz));
    r2 = __dadd_rn(0.0, r2);
    double r2s = __dadd_rn(r2, eps2);
    if (r2s == 0.0) return;
    double f = __ddiv_rn(__dmul_rn(G, cm.w), __dmul_rn(r2s, __dsqrt_rn(r2s)));
    ax = __dadd_rn(ax, __dmul_rn(f, dx));
    ay = __dadd_rn(ay, __dmul_rn(f, dy));
    if (DIM == 3) az = __dadd_rn(az, __dmul_rn(f, dz));
}

template <int DIM>
__global__ void __launch_bounds__(kTravThreads)
k_traverse_exact(TreeDev t, const double* __restrict__ tx, const double* __restrict__ ty,
                 const double* __restrict__ tz, const int32_t* __restrict__ self_id,
                 const int32_t* __restrict__ out_idx, int64_t nt, double theta, double eps,
                 double G, double* __restrict__ out, unsigned* __restrict__ err,
                 unsigned long long* __restrict__ stats)
{
    __shared__ int2 stack[kTravWarps][kStackDepth];
    __shared__ double px[kTravWarps][kWarp], py[kTravWarps][kWarp], pz[kTravWarps][kWarp],
        pm[kTravWarps][kWarp];
    __shared__ int32_t pid[kTravWarps][kWarp];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const double eps2 = __dmul_rn(eps, eps);
    const unsigned FULL = 0xffffffffu;

    for (int64_t base = ((int64_t)blockIdx.x * kTravWarps + w) * kWarp; base < nt;
         base += (int64_t)gridDim.x * kTravWarps * kWarp) {
        const int64_t i = base + lane;
        const bool valid = i < nt;
        const double x = valid ? tx[i] : 0.0, y = valid ? ty[i] : 0.0;
        const double z = (valid && DIM == 3) ? tz[i] : 0.0;
        const int32_t me = (valid && self_id) ? self_id[i] : -1;
        double ax = 0.0, ay = 0.0, az = 0.0;
        unsigned long long n_p2p = 0, n_m2p = 0, n_visit = 0;
        const unsigned live = __ballot_sync(FULL, valid);
        if (lane == 0) stack[w][0] = make_int2(0, (int)live);
        int sp = 1;
        bool overflow = false;
        __syncwarp();
        while (sp > 0) {
            const int2 e = stack[w][--sp];
            __syncwarp();
            const int node = e.x;
            const unsigned mask = (unsigned)e.y;
            const bool act = (mask >> lane) & 1u;
            n_visit += act;
            const NodeCM cm = t.cm[node];
            if (cm.w == 0.0) continue;                       // bh.py:514
            const int fc = t.first_child[node];
            if (fc < 0) {                                    // leaf: bh.py:520-524
                const int s = t.start[node], c = t.count[node];
                double lx = 0.0, ly = 0.0, lz = 0.0;
                for (int b = 0; b < c; b += kWarp) {
                    const int jj = b + lane;
                    if (jj < c) {
                        px[w][lane] = t.sx[s + jj];
                        py[w][lane] = t.sy[s + jj];
                        if (DIM == 3) pz[w][lane] = t.sz[s + jj];
                        pm[w][lane] = t.sm[s + jj];
                        pid[w][lane] = t.perm[s + jj];
                    }
                    __syncwarp();
                    const int cnt = min(kWarp, c - b);
                    if (act) {
                        for (int q = 0; q < cnt; q++) {
                            if (pid[w][q] == me) continue;   // self skip, bh.py:254
                            const double dx = __dsub_rn(px[w][q], x);
                            const double dy = __dsub_rn(py[w][q], y);
                            const double dz = DIM == 3 ? __dsub_rn(pz[w][q], z) : 0.0;
                            double r2 = __dmul_rn(dx, dx);
                            r2 = __dadd_rn(r2, __dmul_rn(dy, dy));
                            if (DIM == 3) r2 = __dadd_rn(r2, __dmul_rn(dz, dz));
                            r2 = __dadd_rn(r2, eps2);
                            if (r2 == 0.0) continue;
                            const double ri = __ddiv_rn(1.0, __dsqrt_rn(r2));
                            const double ri3 = __dmul_rn(__dmul_rn(ri, ri), ri);
                            const double f = __dmul_rn(__dmul_rn(G, pm[w][q]), ri3);
                            lx = __dadd_rn(lx, __dmul_rn(f, dx));
                            ly = __dadd_rn(ly, __dmul_rn(f, dy));
                            if (DIM == 3) lz = __dadd_rn(lz, __dmul_rn(f, dz));
                            n_p2p++;
                        }
                    }
                    __syncwarp();
                }
                if (act) {
                    ax = __dadd_rn(ax, lx);
                    ay = __dadd_rn(ay, ly);
                    az = __dadd_rn(az, lz);
                }
            } else {                                         // internal: bh.py:525-546
                bool open = false;
                if (act) open = open_exact<DIM>(x, y, z, cm, t.size[node], theta);
                const unsigned omask = __ballot_sync(FULL, act && open);
                if (act && !open) {
                    monopole_exact<DIM>(x, y, z, cm, eps2, G, ax, ay, az);
                    n_m2p++;
                }
                if (omask) {
                    if (sp + 2 > kStackDepth) { overflow = true; break; }
                    if (lane == 0) {
                        stack[w][sp] = make_int2(fc, (int)omask);        // left pushed first
                        stack[w][sp + 1] = make_int2(fc + 1, (int)omask); // right pops first
                    }
                    sp += 2;
                    __syncwarp();
                }
            }
        }
        if (overflow && lane == 0) atomicOr(err, kErrStackOverflow);
        if (stats) {
            for (int o = 16; o > 0; o >>= 1) {
                n_p2p += __shfl_down_sync(FULL, n_p2p, o);
                n_m2p += __shfl_down_sync(FULL, n_m2p, o);
                n_visit += __shfl_down_sync(FULL, n_visit, o);
            }
            if (lane == 0) {
                atomicAdd(&stats[0], n_p2p);
                atomicAdd(&stats[1], n_m2p);
                atomicAdd(&stats[2], n_visit);
            }
        }
        if (valid) {
            const int64_t o = out_idx ? out_idx[i] : i;
            out[o * DIM] = ax;
            out[o * DIM + 1] = ay;
            if (DIM == 3) out[o * DIM + 2] = az;
        }
    }
}

// FP64 direct sum (the theta = 0 limit of the reference; pair arithmetic of
// bh.py:262-278).  Targets given as AoS; self_id[i] >= 0 excludes that
// source.  Sources are staged through shared memory in tiles.  Block
// (x, y) handles targets [256x, 256x + 256) against source chunk y; with
// more than one chunk, per-chunk partial sums go to `partial` and
// k_direct_reduce adds them in chunk order (deterministic).
constexpr int kDirectThreads = 256;

template <int DIM>
__global__ void __launch_bounds__(kDirectThreads)
k_direct(const double* __restrict__ pos, const double* __restrict__ mass, int64_t n,
         const double* __restrict__ targets, const int64_t* __restrict__ self_id, int64_t nt,
         double eps, double G, int64_t chunk, double* __restrict__ out)
{
    __shared__ double sx[kDirectThreads], sy[kDirectThreads], sz[kDirectThreads],
        sm[kDirectThreads];
    const int64_t i = blockIdx.x * (int64_t)kDirectThreads + threadIdx.x;
    const bool valid = i < nt;
    const int64_t me = (valid && self_id) ? self_id[i] : -1;
    double x = 0.0, y = 0.0, z = 0.0;
    if (valid) {
        const double* p = self_id ? pos + me * DIM : targets + i * DIM;
        x = p[0];
        y = p[1];
        if (DIM == 3) z = p[2];
    }
    const double eps2 = __dmul_rn(eps, eps);
    double ax = 0.0, ay = 0.0, az = 0.0;
    const int64_t j0 = (int64_t)blockIdx.y * chunk;
    const int64_t j1 = j0 + chunk < n ? j0 + chunk : n;
    for (int64_t b = j0; b < j1; b += kDirectThreads) {
        const int64_t j = b + threadIdx.x;
        __syncthreads();
        if (j < j1) {
            sx[threadIdx.x] = pos[j * DIM];
            sy[threadIdx.x] = pos[j * DIM + 1];
            sz[threadIdx.x] = DIM == 3 ? pos[j * DIM + 2] : 0.0;
            sm[threadIdx.x] = mass[j];
        }
        __syncthreads();
        const int cnt = (int)((j1 - b) < kDirectThreads ? (j1 - b) : kDirectThreads);
        if (valid) {
            for (int q = 0; q < cnt; q++) {
                if (b + q == me) continue;
                const double dx = __dsub_rn(sx[q], x), dy = __dsub_rn(sy[q], y);
                const double dz = DIM == 3 ? __dsub_rn(sz[q], z) : 0.0;
                double r2 = __dmul_rn(dx, dx);
                r2 = __dadd_rn(r2, __dmul_rn(dy, dy));
                if (DIM == 3) r2 = __dadd_rn(r2, __dmul_rn(dz, dz));
                r2 = __dadd_rn(r2, eps2);
                if (r2 == 0.0) continue;
                const double ri = __ddiv_rn(1.0, __dsqrt_rn(r2));
                const double f = __dmul_rn(__dmul_rn(G, sm[q]), __dmul_rn(__dmul_rn(ri, ri), ri));
                ax = __dadd_rn(ax, __dmul_rn(f, dx));
                ay = __dadd_rn(ay, __dmul_rn(f, dy));
                if (DIM == 3) az = __dadd_rn(az, __dmul_rn(f, dz));
            }
        }
    }
    if (valid) {
        double* o = out + ((int64_t)blockIdx.y * nt + i) * DIM;
        o[0] = ax;
        o[1] = ay;
        if (DIM == 3) o[2] = az;
    }
}

__global__ void k_direct_reduce(const double* __restrict__ partial, int64_t nt, int dim,
                                int chunks, double* __restrict__ out)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nt * dim;
         k += (int64_t)gridDim.x * blockDim.x) {
        double s = partial[k];
        for (int c = 1; c < chunks; c++) s = __dadd_rn(s, partial[(int64_t)c * nt * dim + k]);
        out[k] = s;
    }
}

int launch_traverse_exact(const TreeDev& t, const double* tx, const double* ty, const double* tz,
                          const int32_t* self_id, const int32_t* out_idx, int64_t nt, double theta,
                          double eps, double G, double* out, unsigned* err,
                          unsigned long long* stats, cudaStream_t s)
{
    if (nt <= 0) return kOk;
    int64_t warps = (nt + kWarp - 1) / kWarp;
    unsigned grid = grid_for(warps, kTravWarps, 152u * 64u);
    if (t.dim == 3)
        k_traverse_exact<3><<<grid, kTravThreads, 0, s>>>(t, tx, ty, tz, self_id, out_idx, nt, theta,
                                                         eps, G, out, err, stats);
    else
        k_traverse_exact<2><<<grid, kTravThreads, 0, s>>>(t, tx, ty, tz, self_id, out_idx, nt, theta,
                                                         eps, G, out, err, stats);
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    return kOk;
}

// ---------------------------------------------------------------------------
// Operation counts of compute_tree_statistics (bhut/traverse/bh.py:604-700)
// over any TreeData arrays: per target, nodes popped (empty and out-of-range
// ones included), count - 1 particles for every visited non-empty leaf, and
// accepted internal nodes; opening test of bh.py:576-601 (open_exact).
// One thread per target, private stack; totals summed with warp shuffles and
// one 64-bit atomic per warp and counter.
// ---------------------------------------------------------------------------
constexpr int kStatStack = 128;

template <int DIM>
__global__ void __launch_bounds__(256)
k_tree_statistics(StatTree t, const double* __restrict__ tg, int64_t nt, double theta,
                  unsigned long long* __restrict__ totals, unsigned* __restrict__ err)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    unsigned long long nodes = 0, parts = 0, monos = 0;
    if (i < nt) {
        const double x = tg[i * DIM], y = tg[i * DIM + 1], z = DIM == 3 ? tg[i * DIM + 2] : 0.0;
        int64_t stack[kStatStack];
        int sp = 0;
        stack[sp++] = 0;
        while (sp > 0) {
            const int64_t k = stack[--sp];
            nodes++;
            if (k < 0 || k >= t.m || t.mass[k] == 0.0) continue;
            const int64_t fc = t.first_child[k];
            if (fc == -1) {
                const int64_t c = t.count[k];
                if (t.start[k] != -1 && c > 0) parts += (unsigned long long)(c - 1);
                continue;
            }
            NodeCM cm;
            cm.x = t.com[k * DIM];
            cm.y = t.com[k * DIM + 1];
            cm.z = DIM == 3 ? t.com[k * DIM + 2] : 0.0;
            cm.w = 0.0;
            if (open_exact<DIM>(x, y, z, cm, __dmul_rn(2.0, t.half_size[k]), theta)) {
                const int64_t nc = t.child_count[k];
                if (sp + nc > kStatStack) {
                    atomicOr(err, kErrStackOverflow);
                    break;
                }
                for (int64_t j = 0; j < nc; j++) stack[sp++] = fc + j;
            } else {
                monos++;
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        nodes += __shfl_down_sync(0xffffffffu, nodes, o);
        parts += __shfl_down_sync(0xffffffffu, parts, o);
        monos += __shfl_down_sync(0xffffffffu, monos, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&totals[0], nodes);
        atomicAdd(&totals[1], parts);
        atomicAdd(&totals[2], monos);
    }
}

int launch_tree_statistics(const StatTree& t, int dim, const double* targets, int64_t nt,
                           double theta, unsigned long long* totals, unsigned* err,
                           cudaStream_t s)
{
    BHUT_CUDA(cudaMemsetAsync(totals, 0, sizeof(unsigned long long) * 3, s));
    if (nt <= 0) return kOk;
    const unsigned grid = (unsigned)((nt + 255) / 256);
    if (dim == 3) k_tree_statistics<3><<<grid, 256, 0, s>>>(t, targets, nt, theta, totals, err);
    else k_tree_statistics<2><<<grid, 256, 0, s>>>(t, targets, nt, theta, totals, err);
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    return kOk;
}

int direct_chunks(int64_t n, int64_t nt)
{
    const int64_t tblocks = (nt + kDirectThreads - 1) / kDirectThreads;
    int64_t want = (152 * 8 + tblocks - 1) / tblocks;        // fill the GPU ~8 blocks per SM
    int64_t maxc = (n + 4095) / 4096;                         // at least 4096 sources a chunk
    int64_t c = want < maxc ? want : maxc;
    return (int)(c < 1 ? 1 : (c > 1024 ? 1024 : c));
}

int launch_direct(const double* pos, const double* mass, int64_t n, int dim, const double* targets,
                  const int64_t* self_id, int64_t nt, double eps, double G, double* out,
                  double* partial, int chunks, cudaStream_t s)
{
    if (nt <= 0) return kOk;
    const int64_t chunk = (n + chunks - 1) / chunks;
    dim3 grid((unsigned)((nt + kDirectThreads - 1) / kDirectThreads), (unsigned)chunks);
    double* dst = chunks > 1 ? partial : out;
    if (dim == 3)
        k_direct<3><<<grid, kDirectThreads, 0, s>>>(pos, mass, n, targets, self_id, nt, eps, G, chunk,
                                                    dst);
    else
        k_direct<2><<<grid, kDirectThreads, 0, s>>>(pos, mass, n, targets, self_id, nt, eps, G, chunk,
                                                    dst);
    if (chunks > 1)
        k_direct_reduce<<<grid_for(nt * dim, 256), 256, 0, s>>>(partial, nt, dim, chunks, out);
    BHUT_CUDA(cudaGetLastError());
    note_launches(chunks > 1 ? 2 : 1);
    return kOk;
}

}  // namespace bhut
