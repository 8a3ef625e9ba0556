// Shared definitions for the GB300 Barnes-Hut engine (sm_103a).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace bhut {

// Status codes returned through the C ABI (include/bhut_gb300.h).
enum Status : int {
    kOk = 0,
    kInvalid = 1,        // bad argument (maps to ValueError)
    kNotBuilt = 2,       // tree not built
    kCuda = 3,           // CUDA runtime error
    kNoMemory = 4,       // device allocation failed
    kDeviceFlag = 5,     // a kernel raised its error word (stack overflow, ...)
    kInternal = 6,
};

// Error word bits written by kernels (never a trap).
enum DeviceError : unsigned {
    kErrStackOverflow = 1u,
    kErrNonFinite = 2u,
    kErrBadNode = 4u,
    kErrScratchSize = 8u,
};

constexpr int kWarp = 32;
constexpr int kStackDepth = 64;     // per-warp traversal stack entries

void set_error(const char* fmt, ...);
// Counts kernel launches made by the library (reported by bhut_launch_count).
void note_launches(long long k);
int cuda_status(cudaError_t e, const char* what);

#define BHUT_CUDA(call)                                              \
    do {                                                             \
        cudaError_t e__ = (call);                                    \
        if (e__ != cudaSuccess) return ::bhut::cuda_status(e__, #call); \
    } while (0)

#define BHUT_TRY(call)                     \
    do {                                   \
        int s__ = (call);                  \
        if (s__ != ::bhut::kOk) return s__; \
    } while (0)

inline unsigned grid_for(int64_t n, int block, unsigned cap = 152u * 16u)
{
    int64_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (unsigned)g;
}

// ---------------------------------------------------------------------------
// Radix sort of (uint64 key, int32 value) pairs, stable, LSD, 8-bit digits
// (sort.cu).
// ---------------------------------------------------------------------------
// Keys per tile: 2^BHUT_SORT_TILE_SHIFT (8 warps x 256 keys by default).
// Smaller tiles give more blocks for the latency-bound rank/scatter step at
// moderate n, at the price of larger count tables.
#ifndef BHUT_SORT_TILE_SHIFT
#define BHUT_SORT_TILE_SHIFT 11
#endif
constexpr int kSortTileShift = BHUT_SORT_TILE_SHIFT;
constexpr int kSortTile = 1 << kSortTileShift;
constexpr int kSortThreads = 256;
constexpr int kSortPassesMax = 8;      // 64 key bits

constexpr int64_t sort_tiles(int64_t n) { return (n + kSortTile - 1) / kSortTile; }
constexpr size_t sort_align(size_t x) { return (x + 255) & ~(size_t)255; }
// Scratch of radix_sort_pairs for n keys: the ping-pong keys and values, two
// bucket-major count tables (256 x tiles) and the per-pass digit totals.
constexpr size_t sort_scratch_bytes(int64_t n)
{
    return sort_align(sizeof(uint64_t) * (size_t)n) + sort_align(sizeof(int32_t) * (size_t)n) +
           2 * sort_align(sizeof(uint32_t) * 256 * (size_t)sort_tiles(n)) +
           sort_align(sizeof(uint32_t) * 256 * kSortPassesMax);
}
// Sorts keys[0..n) ascending with values carried along.  `bits` is the
// number of low key bits that can be non-zero (passes = ceil(bits / 8)).
// The result ends in keys/vals.  Scratch must hold sort_scratch_bytes(n).
int radix_sort_pairs(uint64_t* keys, int32_t* vals, int64_t n, int bits, void* scratch,
                     cudaStream_t stream);

}  // namespace bhut
