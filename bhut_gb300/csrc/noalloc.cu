// Morton argsort that allocates no device memory.
//
// Some callers of this library cannot call cudaMalloc: processes whose GPU
// memory is owned by another allocator (a framework that reserves most of
// HBM up front, so a foreign cudaMalloc fails or fragments its pool), and
// time-critical step loops in which cudaMalloc/cudaFree would synchronize the
// device.  bhut_morton_argsort_noalloc serves them: it runs the same bounding
// box, Morton-key and stable radix-sort kernels as bhut_morton_argsort, but
// every scratch byte (sort ping-pong buffers, digit counts, scan partials,
// bounding-box partials, counters) lives in one file-scope __device__ array
// of fixed size.  The caller still provides the inputs and outputs.
//
// Limits and sharing:
//  * at most kNoAllocMaxPoints points per call (the array is sized for it);
//    larger requests are rejected with BHUT_EINVAL;
//  * the array (about 13.7 MB) is held on every GPU that loads this library
//    until the process exits;
//  * every call uses the same array and leaves its contents behind; the
//    counters that must start at zero are cleared at the start of each call.
//    Calls whose work overlaps on the GPU (different streams or threads at
//    the same time) race on the array and must not be issued;
//  * the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress, once per device, with that device current); make
//    that first call before any stream capture.  The address is kept for the
//    life of the process, so a process that calls cudaDeviceReset must not
//    call this entry point again afterwards;
//  * each call ends by reading the error word back and synchronizing its
//    stream, so a bad input is reported by the call that received it.
#include <mutex>

#include "../../include/bhut_gb300.h"
#include "tree.cuh"

using namespace bhut;

namespace {

constexpr int64_t kNoAllocMaxPoints = 1 << 20;          // 1,048,576 points
constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
// Region sizes: the sort's scratch for kNoAllocMaxPoints keys, then the
// bounding-box partials, the box and the counters.
constexpr size_t kSortBytes = sort_scratch_bytes(kNoAllocMaxPoints);
constexpr size_t kBoxPartialBytes = align256(sizeof(double) * kBoxPartialDoubles);
constexpr size_t kBoxBytes = 256;
constexpr size_t kWordBytes = 256;                      // counters[8] + error word
constexpr size_t kScratchBytes = kSortBytes + kBoxPartialBytes + kBoxBytes + kWordBytes;

// The scratch array.  Host code must not pass its name to a kernel (on the
// host it is only a stand-in symbol); it uses the device address looked up
// below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (looked up once
// per device).
int scratch_address(void** out)
{
    int dev = 0;
    BHUT_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("device ordinal %d out of range for the no-allocation scratch", dev);
        return kInvalid;
    }
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return cuda_status(e, "cudaGetSymbolAddress(no-allocation scratch)");
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return kOk;
}

// True when p is device memory of device `dev` or managed memory.  Kernels
// here dereference the caller's pointers directly, so memory of another GPU
// (reachable only with peer access) is refused rather than faulted on.
bool on_device(const void* p, int dev)
{
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == dev;
}

}  // namespace

extern "C" int bhut_morton_argsort_noalloc(const double* positions, int64_t n, int dim,
                                           uint64_t* sorted_keys, int32_t* perm, void* stream)
{
    if (dim != 2 && dim != 3) { set_error("dim must be 2 or 3, got %d", dim); return kInvalid; }
    if (n <= 0) { set_error("points array cannot be empty"); return kInvalid; }
    if (n > kNoAllocMaxPoints) {
        set_error("n = %lld exceeds the %lld-point limit of the no-allocation scratch; "
                  "use bhut_morton_argsort", (long long)n, (long long)kNoAllocMaxPoints);
        return kInvalid;
    }
    int dev = 0;
    BHUT_CUDA(cudaGetDevice(&dev));
    if (!on_device(positions, dev) || !on_device(sorted_keys, dev) || !on_device(perm, dev)) {
        set_error("bhut_morton_argsort_noalloc needs device pointers of the current device "
                  "(%d) or managed memory for positions, sorted_keys and perm", dev);
        return kInvalid;
    }
    if (sort_scratch_bytes(n) > kSortBytes) {
        set_error("internal: sort scratch for n = %lld exceeds the reserved region", (long long)n);
        return kInternal;
    }
    void* base = nullptr;
    BHUT_TRY(scratch_address(&base));
    cudaStream_t s = (cudaStream_t)stream;
    char* p = (char*)base;
    void* sort_region = p;
    double* box_partial = (double*)(p + kSortBytes);
    double* box = (double*)(p + kSortBytes + kBoxPartialBytes);
    unsigned* words = (unsigned*)(p + kSortBytes + kBoxPartialBytes + kBoxBytes);
    unsigned* counter = words;        // bbox last-block counter
    unsigned* err = words + 8;        // error word
    BHUT_CUDA(cudaMemsetAsync(words, 0, kWordBytes, s));
    BHUT_TRY(launch_bbox(positions, nullptr, n, dim, box_partial, counter, box, err, s));
    BHUT_TRY(launch_morton(positions, n, dim, box, sorted_keys, perm, s));
    BHUT_TRY(radix_sort_pairs(sorted_keys, perm, n, dim == 3 ? 63 : 42, sort_region, s));
    unsigned e = 0;
    BHUT_CUDA(cudaMemcpyAsync(&e, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    BHUT_CUDA(cudaStreamSynchronize(s));
    if (e & kErrNonFinite) {
        set_error("positions must be finite (NaN or Inf found)");
        return kInvalid;
    }
    if (e) {
        set_error("device error word 0x%x in bhut_morton_argsort_noalloc", e);
        return kDeviceFlag;
    }
    return kOk;
}
