// Stable LSD radix sort of (uint64 key, int32 value) pairs.
//
// Replaces np.argsort(codes, kind='stable') of bhut/utils/morton.py:135.  A
// stable order of the keys is unique, so the permutation is bit-identical to
// numpy's.  8-bit digits; keys are cut into tiles of kSortTile consecutive
// positions (of the order the pass reads).
//
//   k_sort_prep      one read of the keys: every pass's global digit totals
//                    (the totals do not depend on the order) and the first
//                    pass's per-tile digit counts.
//   per pass:
//   k_sort_scan      one block per digit: exclusive scan of that digit's
//                    counts over the tiles, plus the digit's global base
//                    (exclusive prefix of the totals) -> each tile's output
//                    offset for each digit, in stable (tile) order.  Clears
//                    the count table that the scatter below fills.
//   k_sort_scatter   one block per tile: stable rank of every key within the
//                    tile (ballot-based warp multi-split in position order,
//                    warps combined by a per-digit prefix), the tile
//                    reordered by digit in shared memory, then written out in
//                    digit runs, so that consecutive threads store
//                    consecutive addresses.  While writing, it counts the
//                    next pass's digit per destination tile (warp-aggregated
//                    global atomics): the next pass needs no histogram launch.
//
// No block waits on another block (no look-back): the only cross-block
// dependencies are between launches.  Two launches per pass.
#include <atomic>

#include "common.cuh"

namespace bhut {

namespace {

constexpr int kItems = kSortTile / kSortThreads;       // keys per thread
constexpr int kWarpsPerTile = kSortThreads / kWarp;    // 8
constexpr int kWarpSpan = kSortTile / kWarpsPerTile;   // keys per warp
constexpr int kScanThreads = 256;
constexpr int kTileShift = kSortTileShift;             // log2(kSortTile)
static_assert(kItems >= 1 && kItems * kSortThreads == kSortTile, "tile of whole warps");
// resident scatter blocks per SM the register budget must allow (shared
// memory allows three 59 KB tiles of 4,096 keys, five 34 KB tiles of 2,048)
constexpr int kScatterMinBlocks = kSortTileShift >= 12 ? 3 : 4;
static_assert(kScanThreads == kSortThreads, "the scan helper serves both kernels");

__device__ __forceinline__ int64_t item_pos(int64_t tile, int warp, int item, int lane)
{
    return tile * kSortTile + (int64_t)warp * kWarpSpan + item * kWarp + lane;
}

// Shared memory of the scatter kernel.
struct ScatterSmem {
    uint64_t keys[kSortTile];
    int32_t vals[kSortTile];
    uint32_t warp_counts[kWarpsPerTile][256];
    uint32_t delta[256];      // global offset of the digit minus its local offset
    uint32_t local_off[256];
};

// k_sort_prep: block t reads tile t; per-tile counts of digit 0 and the
// global totals of every pass's digit.
__global__ void __launch_bounds__(kSortThreads)
k_sort_prep(const uint64_t* __restrict__ keys, int64_t n, int passes,
            uint32_t* __restrict__ counts0, int64_t tiles, uint32_t* __restrict__ totals)
{
    __shared__ uint32_t hist[kSortPassesMax][256];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t tile = blockIdx.x;
    for (int p = 0; p < passes; p++) hist[p][tid] = 0;
    __syncthreads();
    // shared-memory atomics; a digit that all lanes of the warp share (ties,
    // or the few distinct high digits of clustered keys) is added once
#pragma unroll 4
    for (int i = 0; i < kItems; i++) {
        const int64_t pos = item_pos(tile, warp, i, lane);
        const bool valid = pos < n;
        const unsigned vmask = __ballot_sync(0xffffffffu, valid);
        // (a lane past the end borrows the tile's first key, which exists)
        const uint64_t k = keys[valid ? pos : tile * kSortTile];
        for (int p = 0; p < passes; p++) {
            const unsigned d = (unsigned)(k >> (8 * p)) & 0xFFu;
            const bool same = __all_sync(0xffffffffu, d == __shfl_sync(0xffffffffu, d, 0));
            if (same) {
                if (lane == 0) atomicAdd(&hist[p][d], (unsigned)__popc(vmask));
            } else if (valid) {
                atomicAdd(&hist[p][d], 1u);
            }
        }
    }
    __syncthreads();
    counts0[(int64_t)tid * tiles + tile] = hist[0][tid];
    for (int p = 0; p < passes; p++) {
        const uint32_t c = hist[p][tid];
        if (c) atomicAdd(&totals[p * 256 + tid], c);
    }
}

// Block-wide exclusive scan of one value per thread (kScanThreads threads).
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total,
                                                         uint32_t* warp_sums)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = lane < kScanThreads / kWarp ? warp_sums[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < kScanThreads / kWarp) warp_sums[lane] = s;
    }
    __syncthreads();
    const uint32_t prefix = (warp > 0 ? warp_sums[warp - 1] : 0u) + x - v;
    if (total) *total = warp_sums[kScanThreads / kWarp - 1];
    __syncthreads();
    return prefix;
}

// k_sort_scan: block d turns row d of the count table (bucket-major: digit d
// of tile t is entry d * tiles + t) into output offsets, and clears row d of
// the next pass's table.
__global__ void __launch_bounds__(kScanThreads)
k_sort_scan(uint32_t* __restrict__ counts, int64_t tiles, const uint32_t* __restrict__ totals,
            uint32_t* __restrict__ next_counts)
{
    __shared__ uint32_t warp_sums[kScanThreads / kWarp];
    __shared__ uint32_t s_base;
    const int d = blockIdx.x, tid = threadIdx.x;
    // base of digit d: sum of the totals of digits below d
    uint32_t below = tid < d ? totals[tid] : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) below += __shfl_down_sync(0xffffffffu, below, o);
    if (tid == 0) s_base = 0;
    __syncthreads();
    if ((tid & 31) == 0 && below) atomicAdd(&s_base, below);
    __syncthreads();
    uint32_t carry = s_base;
    uint32_t* row = counts + (int64_t)d * tiles;
    uint32_t* nrow = next_counts ? next_counts + (int64_t)d * tiles : nullptr;
    for (int64_t base = 0; base < tiles; base += kScanThreads) {
        const int64_t t = base + tid;
        const uint32_t v = t < tiles ? row[t] : 0u;
        uint32_t total;
        const uint32_t ex = block_exclusive_scan(v, &total, warp_sums);
        if (t < tiles) {
            row[t] = carry + ex;
            if (nrow) nrow[t] = 0u;
        }
        carry += total;
    }
}

// k_sort_scatter: see the file comment.  `next_counts` (may be null) gets
// the digit at `next_shift` of every key, per destination tile.
__global__ void __launch_bounds__(kSortThreads, kScatterMinBlocks)
k_sort_scatter(const uint64_t* __restrict__ keys_in, const int32_t* __restrict__ vals_in,
               uint64_t* __restrict__ keys_out, int32_t* __restrict__ vals_out, int64_t n,
               int shift, const uint32_t* __restrict__ offsets, int64_t tiles,
               uint32_t* __restrict__ next_counts, int next_shift)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ScatterSmem& sm = *reinterpret_cast<ScatterSmem*>(smem_raw);
    __shared__ uint32_t warp_sums[kSortThreads / kWarp];
    const unsigned FULL = 0xffffffffu;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t tile = blockIdx.x;
#pragma unroll
    for (int w = 0; w < kWarpsPerTile; w++) sm.warp_counts[w][tid] = 0;
    __syncthreads();

    uint64_t k[kItems];
    uint32_t rank[kItems];
    const unsigned lt_mask = (1u << lane) - 1u;
#pragma unroll
    for (int i = 0; i < kItems; i++) {
        const int64_t p = item_pos(tile, warp, i, lane);
        const bool valid = p < n;
        k[i] = valid ? keys_in[p] : ~0ull;
        const unsigned d = (unsigned)(k[i] >> shift) & 0xFFu;
        // lanes holding the same digit (warp multi-split by eight ballots)
        unsigned peers = __ballot_sync(FULL, valid);
#pragma unroll
        for (int b = 0; b < 8; b++) {
            const bool bit = (d >> b) & 1u;
            const unsigned bal = __ballot_sync(FULL, bit);
            peers &= bit ? bal : ~bal;
        }
        const uint32_t before = sm.warp_counts[warp][d];
        rank[i] = before + __popc(peers & lt_mask);
        __syncwarp();
        if (valid && (peers & lt_mask) == 0) sm.warp_counts[warp][d] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // per digit (thread tid = digit): prefix over warps, then the tile-local
    // digit offsets (exclusive scan over digits)
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < kWarpsPerTile; w++) {
        const uint32_t t = sm.warp_counts[w][tid];
        sm.warp_counts[w][tid] = run;
        run += t;
    }
    const uint32_t loc = block_exclusive_scan(run, nullptr, warp_sums);
    sm.local_off[tid] = loc;
    sm.delta[tid] = offsets[(int64_t)tid * tiles + tile] - loc;
    __syncthreads();
    // reorder the tile by digit in shared memory (stable)
#pragma unroll
    for (int i = 0; i < kItems; i++) {
        const int64_t p = item_pos(tile, warp, i, lane);
        if (p < n) {
            const unsigned d = (unsigned)(k[i] >> shift) & 0xFFu;
            const uint32_t lpos = sm.local_off[d] + sm.warp_counts[warp][d] + rank[i];
            if (lpos < (uint32_t)kSortTile) {   // always true; guards shared memory
                sm.keys[lpos] = k[i];
                sm.vals[lpos] = vals_in[p];    // (read here: fewer live registers)
            }
        }
    }
    __syncthreads();
    // write out in digit runs: position j of the reordered tile goes to
    // delta[digit] + j
    const int64_t cnt = min((int64_t)kSortTile, n - tile * kSortTile);
#pragma unroll 4
    for (int j = tid; j < cnt; j += kSortThreads) {
        const uint64_t key = sm.keys[j];
        const unsigned d = (unsigned)(key >> shift) & 0xFFu;
        const uint32_t dst = sm.delta[d] + (uint32_t)j;
        if (dst >= (uint32_t)n) continue;   // always false; guards the output
        keys_out[dst] = key;
        vals_out[dst] = sm.vals[j];
        if (next_counts) {   // warp-aggregated: one atomic per (digit, tile) in the warp
            const unsigned nd = (unsigned)(key >> next_shift) & 0xFFu;
            const unsigned dtile = dst >> kTileShift;
            const unsigned peers = __match_any_sync(__activemask(), (dtile << 8) | nd);
            if ((peers & ((1u << lane) - 1u)) == 0)
                atomicAdd(&next_counts[(int64_t)nd * tiles + dtile], (unsigned)__popc(peers));
        }
    }
}

struct SortLayout {
    uint64_t* keys_alt;
    int32_t* vals_alt;
    uint32_t* counts[2];
    uint32_t* totals;
};

SortLayout carve(void* scratch, int64_t n)
{
    const int64_t tiles = sort_tiles(n);
    char* s = (char*)scratch;
    SortLayout L;
    L.keys_alt = (uint64_t*)s; s += sort_align(sizeof(uint64_t) * (size_t)n);
    L.vals_alt = (int32_t*)s;  s += sort_align(sizeof(int32_t) * (size_t)n);
    L.counts[0] = (uint32_t*)s; s += sort_align(sizeof(uint32_t) * 256 * (size_t)tiles);
    L.counts[1] = (uint32_t*)s; s += sort_align(sizeof(uint32_t) * 256 * (size_t)tiles);
    L.totals = (uint32_t*)s;
    return L;
}

}  // namespace

int radix_sort_pairs(uint64_t* keys, int32_t* vals, int64_t n, int bits, void* scratch,
                     cudaStream_t stream)
{
    if (n <= 1) return kOk;
    if (n > 0x7fffffffLL) { set_error("radix sort supports at most 2^31-1 keys"); return kInvalid; }
    const int passes = (bits + 7) / 8;
    if (passes < 1 || passes > kSortPassesMax) {
        set_error("radix sort: %d key bits out of range", bits);
        return kInvalid;
    }
    // the scatter's shared memory exceeds the default limit: raise it once
    // per device
    {
        static std::atomic<bool> smem_set[64];
        int dev = 0;
        BHUT_CUDA(cudaGetDevice(&dev));
        if (dev < 0 || dev >= 64 || !smem_set[dev].load(std::memory_order_acquire)) {
            BHUT_CUDA(cudaFuncSetAttribute(k_sort_scatter,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)sizeof(ScatterSmem)));
            // all of the unified L1/shared storage as shared memory (several
            // tiles per SM)
            BHUT_CUDA(cudaFuncSetAttribute(k_sort_scatter,
                                           cudaFuncAttributePreferredSharedMemoryCarveout,
                                           (int)cudaSharedmemCarveoutMaxShared));
            if (dev >= 0 && dev < 64) smem_set[dev].store(true, std::memory_order_release);
        }
    }
    const int64_t tiles = sort_tiles(n);
    const SortLayout L = carve(scratch, n);
    BHUT_CUDA(cudaMemsetAsync(L.totals, 0, sizeof(uint32_t) * 256 * kSortPassesMax, stream));
    k_sort_prep<<<(unsigned)tiles, kSortThreads, 0, stream>>>(keys, n, passes, L.counts[0], tiles,
                                                              L.totals);
    uint64_t *kin = keys, *kout = L.keys_alt;
    int32_t *vin = vals, *vout = L.vals_alt;
    for (int pass = 0; pass < passes; pass++) {
        const bool last = pass + 1 == passes;
        uint32_t* cur = L.counts[pass & 1];
        uint32_t* nxt = last ? nullptr : L.counts[(pass + 1) & 1];
        k_sort_scan<<<256, kScanThreads, 0, stream>>>(cur, tiles, L.totals + 256 * pass, nxt);
        k_sort_scatter<<<(unsigned)tiles, kSortThreads, sizeof(ScatterSmem), stream>>>(
            kin, vin, kout, vout, n, 8 * pass, cur, tiles, nxt, 8 * (pass + 1));
        uint64_t* tk = kin; kin = kout; kout = tk;
        int32_t* tv = vin; vin = vout; vout = tv;
    }
    BHUT_CUDA(cudaGetLastError());
    note_launches(1 + 2ll * passes);
    if (kin != keys) {
        BHUT_CUDA(cudaMemcpyAsync(keys, kin, sizeof(uint64_t) * (size_t)n, cudaMemcpyDeviceToDevice, stream));
        BHUT_CUDA(cudaMemcpyAsync(vals, vin, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToDevice, stream));
    }
    return kOk;
}

}  // namespace bhut
