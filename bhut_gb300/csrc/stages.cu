// Stage kernels behind the reference's module-level functions, and the import
// of a TreeData produced elsewhere into a device tree:
//   k_normalize      space/bbox.py:49-96  normalize_to_unit
//   k_morton_unit    utils/morton.py:48-102  morton_codes (any bits)
//   k_gather_rows    utils/morton.py:139-145  data_arrays[perm]
//   k_import_nodes   TreeData (tree/node.py:15-77) -> device node arrays
//   k_import_perm    int64 perm -> int32, bounds-checked
#include "tree.cuh"

namespace bhut {

__global__ void k_normalize(const double* __restrict__ pts, int64_t n, int dim,
                            const double* __restrict__ pmin, const double* __restrict__ pmax,
                            double top, double* __restrict__ out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n * dim;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int d = (int)(i % dim);
        const double lo = pmin[d], hi = pmax[d];
        const double e0 = __dsub_rn(hi, lo);
        const double extent = e0 <= 0.0 ? 1.0 : e0;      // degenerate axis -> 0.5
        const double offset = e0 <= 0.0 ? 0.5 : 0.0;
        double p = __dadd_rn(__ddiv_rn(__dsub_rn(pts[i], lo), extent), offset);
        p = p > top ? top : p;                             // np.minimum, NaN kept
        out[i] = p;
    }
}

__global__ void k_morton_unit(const double* __restrict__ p01, int64_t n, int dim, int bits,
                              uint64_t* __restrict__ codes, unsigned* __restrict__ bad)
{
    const double scale = ldexp(1.0, bits);
    const uint64_t maxc = (1ull << bits) - 1ull;
    bool out = false;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t c[3] = {0, 0, 0};
        for (int d = 0; d < dim; d++) {
            const double p = p01[i * dim + d];
            out |= (p < 0.0) || (p >= 1.0);
            const uint64_t q = __double2ull_rz(__dmul_rn(p, scale));
            c[d] = q < maxc ? q : maxc;
        }
        codes[i] = dim == 3 ? morton3(c[0], c[1], c[2]) : morton2(c[0], c[1]);
    }
    if (__any_sync(0xffffffffu, out) && (threadIdx.x & 31) == 0) atomicOr(bad, 1u);
}

__global__ void k_gather_rows(const unsigned char* __restrict__ src, int64_t n, int64_t row_bytes,
                              const int64_t* __restrict__ perm, unsigned char* __restrict__ dst,
                              unsigned* __restrict__ err)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n * row_bytes;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = k / row_bytes, b = k - i * row_bytes;
        const int64_t p = perm[i];
        if (p < 0 || p >= n) { atomicOr(err, kErrBadNode); continue; }
        dst[k] = src[p * row_bytes + b];
    }
}

// TreeData arrays (int64 indices, com as (m, dim)) into the device layout:
// int32 first_child/start/count, parent links, (com, mass) records, 2 * half,
// centres; leaves listed for the bottom-up (refit) pass.  Only binary trees
// (child_count 0 or 2, children contiguous) are accepted.
__global__ void k_import_nodes(const int64_t* __restrict__ fc_in, const int64_t* __restrict__ cc_in,
                               const int64_t* __restrict__ st_in, const int64_t* __restrict__ ct_in,
                               const double* __restrict__ half_in, const double* __restrict__ mass_in,
                               const double* __restrict__ com_in, const double* __restrict__ center_in,
                               int64_t m, int64_t n, int dim, int32_t* __restrict__ first_child,
                               int32_t* __restrict__ start, int32_t* __restrict__ count,
                               int32_t* __restrict__ parent, NodeCM* __restrict__ cm,
                               double* __restrict__ size, double* __restrict__ half,
                               double* __restrict__ center, int32_t* __restrict__ leaf_list,
                               unsigned* __restrict__ leaf_counter, unsigned* __restrict__ err)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < m;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t fc = fc_in[k], cc = cc_in[k], st = st_in[k], ct = ct_in[k];
        if (fc == -1) {
            if (cc != 0 || (ct > 0 && (st < 0 || st + ct > n)) || ct < 0) {
                atomicOr(err, kErrBadNode);
                continue;
            }
            const unsigned li = atomicAdd(leaf_counter, 1u);
            if (li < (unsigned)m) leaf_list[li] = (int32_t)k;
        } else {
            if (cc != 2 || fc < 1 || fc + 1 >= m) { atomicOr(err, kErrBadNode); continue; }
            // a node claimed by two parents makes the parent links ambiguous
            if (atomicExch(&parent[fc], (int32_t)k) != -1) atomicOr(err, kErrBadNode);
            if (atomicExch(&parent[fc + 1], (int32_t)k) != -1) atomicOr(err, kErrBadNode);
        }
        first_child[k] = (int32_t)fc;
        start[k] = (int32_t)st;
        count[k] = (int32_t)ct;
        NodeCM c;
        c.x = com_in[k * dim];
        c.y = com_in[k * dim + 1];
        c.z = dim == 3 ? com_in[k * dim + 2] : 0.0;
        c.w = mass_in[k];
        cm[k] = c;
        half[k] = half_in[k];
        size[k] = __dmul_rn(2.0, half_in[k]);
        for (int d = 0; d < dim; d++) center[k * dim + d] = center_in[k * dim + d];
    }
}

__global__ void k_import_perm(const int64_t* __restrict__ in, int64_t n, int32_t* __restrict__ out,
                              unsigned* __restrict__ err)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = in[i];
        if (p < 0 || p >= n) { atomicOr(err, kErrBadNode); out[i] = 0; continue; }
        out[i] = (int32_t)p;
    }
}

__global__ void k_iota(int32_t* __restrict__ out, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (int32_t)i;
}

__global__ void k_widen_i32(const int32_t* __restrict__ in, int64_t n, int64_t* __restrict__ out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = in[i];
}

int launch_iota(int32_t* out, int64_t n, cudaStream_t s)
{
    k_iota<<<grid_for(n, 256), 256, 0, s>>>(out, n);
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    return kOk;
}

int launch_widen_i32(const int32_t* in, int64_t n, int64_t* out, cudaStream_t s)
{
    k_widen_i32<<<grid_for(n, 256), 256, 0, s>>>(in, n, out);
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    return kOk;
}

// Non-finite check of n doubles (and, optionally, m more): flag <- 1.
int launch_normalize(const double* pts, int64_t n, int dim, const double* pmin, const double* pmax,
                     double top, double* out, cudaStream_t s)
{
    k_normalize<<<grid_for(n * dim, 256), 256, 0, s>>>(pts, n, dim, pmin, pmax, top, out);
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    return kOk;
}

int launch_morton_unit(const double* p01, int64_t n, int dim, int bits, uint64_t* codes,
                       unsigned* bad, cudaStream_t s)
{
    k_morton_unit<<<grid_for(n, 256), 256, 0, s>>>(p01, n, dim, bits, codes, bad);
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    return kOk;
}

int launch_gather_rows(const void* src, int64_t n, int64_t row_bytes, const int64_t* perm,
                       void* dst, unsigned* err, cudaStream_t s)
{
    if (n <= 0 || row_bytes <= 0) return kOk;
    k_gather_rows<<<grid_for(n * row_bytes, 256), 256, 0, s>>>(
        (const unsigned char*)src, n, row_bytes, perm, (unsigned char*)dst, err);
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    return kOk;
}

int launch_import_nodes(const int64_t* fc, const int64_t* cc, const int64_t* st, const int64_t* ct,
                        const double* half_in, const double* mass_in, const double* com_in,
                        const double* center_in, int64_t m, int64_t n, int dim,
                        int32_t* first_child, int32_t* start, int32_t* count, int32_t* parent,
                        NodeCM* cm, double* size, double* half, double* center,
                        int32_t* leaf_list, unsigned* leaf_counter, unsigned* err, cudaStream_t s)
{
    BHUT_CUDA(cudaMemsetAsync(parent, 0xff, sizeof(int32_t) * (size_t)m, s));   // -1: root
    BHUT_CUDA(cudaMemsetAsync(leaf_counter, 0, sizeof(unsigned), s));
    k_import_nodes<<<grid_for(m, 256), 256, 0, s>>>(fc, cc, st, ct, half_in, mass_in, com_in,
                                                    center_in, m, n, dim, first_child, start,
                                                    count, parent, cm, size, half, center,
                                                    leaf_list, leaf_counter, err);
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    return kOk;
}

int launch_import_perm(const int64_t* in, int64_t n, int32_t* out, unsigned* err, cudaStream_t s)
{
    k_import_perm<<<grid_for(n, 256), 256, 0, s>>>(in, n, out, err);
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    return kOk;
}

}  // namespace bhut

// ---------------------------------------------------------------------------
// FP32 pipe peak: independent FMA chains (16 per thread), the denominator of
// the FP32-pipe rooflines next to the cuBLAS SGEMM figure.
// ---------------------------------------------------------------------------
namespace bhut {

__global__ void k_fma_peak(float* __restrict__ out, int iters, float m, float c)
{
    float a[16];
#pragma unroll
    for (int j = 0; j < 16; j++) a[j] = threadIdx.x * 1e-3f + (float)j;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 16; j++) a[j] = fmaf(a[j], m, c);
    }
    float s = 0.0f;
#pragma unroll
    for (int j = 0; j < 16; j++) s += a[j];
    out[blockIdx.x * (int64_t)blockDim.x + threadIdx.x] = s;
}

int measure_fp32_peak(double* tflops)
{
    int dev = 0, sms = 0;
    BHUT_CUDA(cudaGetDevice(&dev));
    BHUT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 8, threads = 256, iters = 20000;
    float* out = nullptr;
    BHUT_CUDA(cudaMalloc(&out, sizeof(float) * blocks * threads));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int r = 0; r < 3; r++) {
        cudaEventRecord(e0);
        k_fma_peak<<<blocks, threads>>>(out, iters, 0.999f, 1e-3f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (r > 0 && ms < best) best = ms;
    }
    note_launches(3);
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return cuda_status(e, "fp32 peak kernel");
    *tflops = 2.0 * 16.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
    return kOk;
}

}  // namespace bhut
