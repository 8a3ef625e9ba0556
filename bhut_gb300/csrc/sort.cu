// Stable LSD radix sort of (uint64 key, int32 value) pairs.
//
// Replaces np.argsort(codes, kind='stable') of bhut/utils/morton.py:135.  A
// stable order of the keys is unique, so the permutation is bit-identical to
// numpy's.  Each 8-bit pass is three steps:
//   1. per-tile digit histograms        (k_tile_histogram)
//   2. exclusive scan of the bucket-major count table (digit b of tile t is
//      entry b * tiles + t, so one scan yields every tile's output offset in
//      stable order)                     (k_scan_*)
//   3. stable scatter: within a tile, keys are ranked per warp with
//      __match_any_sync in position order, warps are combined by a per-digit
//      prefix over warps                 (k_tile_scatter)
// No step waits on another block, so nothing can spin.
#include "common.cuh"

namespace bhut {

namespace {

constexpr int kItems = kSortTile / kSortThreads;  // 16 keys per thread
constexpr int kWarpsPerTile = kSortThreads / kWarp;
constexpr int kWarpSpan = kSortTile / kWarpsPerTile;  // 512 keys per warp
constexpr int kScanChunk = 4096;                      // entries per scan block
constexpr int kScanThreads = 1024;

__device__ __forceinline__ int64_t item_pos(int64_t tile, int warp, int item, int lane)
{
    return tile * kSortTile + (int64_t)warp * kWarpSpan + item * kWarp + lane;
}

__global__ void __launch_bounds__(kSortThreads)
k_tile_histogram(const uint64_t* __restrict__ keys, int64_t n, int shift,
                 uint32_t* __restrict__ counts, int64_t tiles)
{
    __shared__ uint32_t hist[256];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t tile = blockIdx.x;
    hist[tid] = 0;
    __syncthreads();
#pragma unroll 4
    for (int i = 0; i < kItems; i++) {
        int64_t p = item_pos(tile, warp, i, lane);
        if (p < n) atomicAdd(&hist[(keys[p] >> shift) & 0xFF], 1u);
    }
    __syncthreads();
    counts[(int64_t)tid * tiles + tile] = hist[tid];
}

// Block-level exclusive scan helper over kScanThreads values.
__device__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total)
{
    __shared__ uint32_t warp_sums[kScanThreads / kWarp];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = warp_sums[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        warp_sums[lane] = s;
    }
    __syncthreads();
    uint32_t prefix = (warp > 0 ? warp_sums[warp - 1] : 0u) + x - v;
    if (total) *total = warp_sums[kScanThreads / kWarp - 1];
    __syncthreads();
    return prefix;
}

__global__ void __launch_bounds__(kScanThreads)
k_scan_reduce(const uint32_t* __restrict__ data, int64_t len, uint32_t* __restrict__ block_sums)
{
    const int64_t base = (int64_t)blockIdx.x * kScanChunk;
    uint32_t s = 0;
    for (int i = threadIdx.x; i < kScanChunk; i += kScanThreads) {
        int64_t p = base + i;
        if (p < len) s += data[p];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    __shared__ uint32_t ws[kScanThreads / kWarp];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t t = ws[threadIdx.x];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) block_sums[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(kScanThreads)
k_scan_top(uint32_t* __restrict__ block_sums, int64_t nblocks)
{
    uint32_t carry = 0;
    for (int64_t base = 0; base < nblocks; base += kScanThreads) {
        int64_t p = base + threadIdx.x;
        uint32_t v = p < nblocks ? block_sums[p] : 0u;
        uint32_t total;
        uint32_t ex = block_exclusive_scan(v, &total);
        if (p < nblocks) block_sums[p] = carry + ex;
        carry += total;
    }
}

__global__ void __launch_bounds__(kScanThreads)
k_scan_down(uint32_t* __restrict__ data, int64_t len, const uint32_t* __restrict__ block_sums)
{
    const int64_t base = (int64_t)blockIdx.x * kScanChunk;
    constexpr int per = kScanChunk / kScanThreads;  // 4 consecutive entries per thread
    uint32_t v[per];
    uint32_t local = 0;
#pragma unroll
    for (int j = 0; j < per; j++) {
        int64_t p = base + (int64_t)threadIdx.x * per + j;
        v[j] = p < len ? data[p] : 0u;
        local += v[j];
    }
    uint32_t ex = block_exclusive_scan(local, nullptr) + block_sums[blockIdx.x];
#pragma unroll
    for (int j = 0; j < per; j++) {
        int64_t p = base + (int64_t)threadIdx.x * per + j;
        if (p < len) data[p] = ex;
        ex += v[j];
    }
}

__global__ void __launch_bounds__(kSortThreads)
k_tile_scatter(const uint64_t* __restrict__ keys_in, const int32_t* __restrict__ vals_in,
               uint64_t* __restrict__ keys_out, int32_t* __restrict__ vals_out, int64_t n,
               int shift, const uint32_t* __restrict__ offsets, int64_t tiles)
{
    __shared__ uint32_t warp_counts[kWarpsPerTile][256];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t tile = blockIdx.x;
    for (int w = 0; w < kWarpsPerTile; w++) warp_counts[w][tid] = 0;
    __syncthreads();

    uint64_t k[kItems];
    uint32_t rank[kItems];
    const unsigned lt_mask = (1u << lane) - 1u;
#pragma unroll
    for (int i = 0; i < kItems; i++) {
        int64_t p = item_pos(tile, warp, i, lane);
        bool valid = p < n;
        unsigned vmask = __ballot_sync(0xffffffffu, valid);
        k[i] = valid ? keys_in[p] : 0ull;
        rank[i] = 0;
        if (valid) {
            unsigned d = (unsigned)(k[i] >> shift) & 0xFFu;
            unsigned peers = __match_any_sync(vmask, d);
            uint32_t base = warp_counts[warp][d];
            rank[i] = base + __popc(peers & lt_mask);
            __syncwarp(vmask);
            if ((peers & lt_mask) == 0) warp_counts[warp][d] = base + __popc(peers);
        }
        __syncwarp();
    }
    __syncthreads();
    {   // per-digit exclusive prefix over the warps of this tile
        uint32_t run = 0;
        for (int w = 0; w < kWarpsPerTile; w++) {
            uint32_t t = warp_counts[w][tid];
            warp_counts[w][tid] = run;
            run += t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kItems; i++) {
        int64_t p = item_pos(tile, warp, i, lane);
        if (p < n) {
            unsigned d = (unsigned)(k[i] >> shift) & 0xFFu;
            int64_t dst = (int64_t)offsets[(int64_t)d * tiles + tile] + warp_counts[warp][d] + rank[i];
            keys_out[dst] = k[i];
            vals_out[dst] = vals_in[p];
        }
    }
}

inline size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

int64_t sort_tiles(int64_t n) { return (n + kSortTile - 1) / kSortTile; }

size_t sort_scratch_bytes(int64_t n)
{
    int64_t tiles = sort_tiles(n);
    int64_t len = 256 * tiles;
    int64_t nb = (len + kScanChunk - 1) / kScanChunk;
    return align_up(sizeof(uint64_t) * (size_t)n) + align_up(sizeof(int32_t) * (size_t)n) +
           align_up(sizeof(uint32_t) * (size_t)len) + align_up(sizeof(uint32_t) * (size_t)(nb + 1));
}

int radix_sort_pairs(uint64_t* keys, int32_t* vals, int64_t n, int bits, void* scratch,
                     cudaStream_t stream)
{
    if (n <= 1) return kOk;
    if (n > 0x7fffffffLL) { set_error("radix sort supports at most 2^31-1 keys"); return kInvalid; }
    int64_t tiles = sort_tiles(n);
    int64_t len = 256 * tiles;
    int64_t nb = (len + kScanChunk - 1) / kScanChunk;
    char* s = (char*)scratch;
    uint64_t* keys_alt = (uint64_t*)s; s += align_up(sizeof(uint64_t) * (size_t)n);
    int32_t* vals_alt = (int32_t*)s;   s += align_up(sizeof(int32_t) * (size_t)n);
    uint32_t* counts = (uint32_t*)s;   s += align_up(sizeof(uint32_t) * (size_t)len);
    uint32_t* bsums = (uint32_t*)s;

    int passes = (bits + 7) / 8;
    uint64_t *kin = keys, *kout = keys_alt;
    int32_t *vin = vals, *vout = vals_alt;
    for (int pass = 0; pass < passes; pass++) {
        int shift = pass * 8;
        k_tile_histogram<<<(unsigned)tiles, kSortThreads, 0, stream>>>(kin, n, shift, counts, tiles);
        k_scan_reduce<<<(unsigned)nb, kScanThreads, 0, stream>>>(counts, len, bsums);
        k_scan_top<<<1, kScanThreads, 0, stream>>>(bsums, nb);
        k_scan_down<<<(unsigned)nb, kScanThreads, 0, stream>>>(counts, len, bsums);
        k_tile_scatter<<<(unsigned)tiles, kSortThreads, 0, stream>>>(kin, vin, kout, vout, n, shift,
                                                                     counts, tiles);
        uint64_t* tk = kin; kin = kout; kout = tk;
        int32_t* tv = vin; vin = vout; vout = tv;
    }
    BHUT_CUDA(cudaGetLastError());
    note_launches(5ll * passes);
    if (kin != keys) {
        BHUT_CUDA(cudaMemcpyAsync(keys, kin, sizeof(uint64_t) * (size_t)n, cudaMemcpyDeviceToDevice, stream));
        BHUT_CUDA(cudaMemcpyAsync(vals, vin, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToDevice, stream));
    }
    return kOk;
}

}  // namespace bhut
