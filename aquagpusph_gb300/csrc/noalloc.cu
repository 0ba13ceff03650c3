// aqua_radix_sort_noalloc(): the stable radix sort for callers that must not
// allocate device memory.
//
// Some hosts of this library cannot call cudaMalloc: a tool that runs inside
// another runtime's step loop where every device buffer is owned and sized
// up front by that runtime (as the reference's Variables registry does),
// code running while a stream is being captured into a CUDA graph, or a
// process that works under a fixed device-memory budget.  Such callers get
// a sort that needs no context: its scratch is the file-scope array below,
// which exists on every GPU that loads the library, from load until exit.
//
// Limits and sharing:
//   - at most AQUA_NOALLOC_SORT_MAX_KEYS keys per call (larger sizes are
//     rejected with AQUA_ERR_CAPACITY before anything is launched);
//   - all calls on a device share the one array and it keeps the contents
//     of the last call: calls whose work overlaps on the GPU (different
//     streams without ordering between them) race and give wrong results;
//   - the first call on a device looks the array's device address up
//     (cudaGetSymbolAddress, with that device current) and caches it; make
//     that first call before any stream capture.
#include <cstdio>
#include <mutex>

#include "aqua_internal.cuh"
#include "kernels.cuh"

using namespace aqua;

namespace {

constexpr uint32_t kMaxKeys = AQUA_NOALLOC_SORT_MAX_KEYS;
constexpr uint32_t kMaxBlocks = (kMaxKeys + kSortTile - 1) / kSortTile;
// keys ping-pong partner, values ping-pong pair, per-pass counts, totals
constexpr size_t kWords = 3ull * kMaxKeys + 256ull * kMaxBlocks + 256ull;

static __device__ __align__(256) uint32_t g_sort_scratch[kWords];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
uint32_t* g_scratch[kMaxDevices] = {};

// Device address of g_sort_scratch on the current device (looked up once)
aqua_status
scratch_for_current_device(uint32_t** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return AQUA_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_sort_scratch);
        if (e != cudaSuccess || p == nullptr) {
            std::fprintf(stderr, "aqua_radix_sort_noalloc: cudaGetSymbolAddress "
                                 "failed: %s\n", cudaGetErrorString(e));
            return AQUA_ERR_CUDA;
        }
        g_scratch[dev] = static_cast<uint32_t*>(p);
    }
    *out = g_scratch[dev];
    return AQUA_OK;
}

#define NA_CUDA(call)                                                          \
    do {                                                                       \
        const cudaError_t e_ = (call);                                         \
        if (e_ != cudaSuccess) {                                               \
            std::fprintf(stderr, "aqua_radix_sort_noalloc: %s failed: %s\n",   \
                         #call, cudaGetErrorString(e_));                       \
            return AQUA_ERR_CUDA;                                              \
        }                                                                      \
    } while (0)

}  // namespace

extern "C" aqua_status
aqua_radix_sort_noalloc(uint32_t* keys, uint32_t* perm, uint32_t* inv_perm,
                        uint32_t n, uint32_t key_bits, void* stream)
{
    if (!keys || key_bits > 32)
        return AQUA_ERR_INVALID;
    if (n > kMaxKeys) {
        std::fprintf(stderr, "aqua_radix_sort_noalloc: %u keys exceed the "
                             "maximum of %u\n", n, kMaxKeys);
        return AQUA_ERR_CAPACITY;
    }
    if (n == 0)
        return AQUA_OK;
    uint32_t* base = nullptr;
    const aqua_status st = scratch_for_current_device(&base);
    if (st != AQUA_OK)
        return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the caller's keys are one half of the key ping-pong (sorted in place)
    uint32_t* kbuf[2] = { keys, base };
    uint32_t* vbuf[2] = { base + kMaxKeys, base + 2ull * kMaxKeys };
    uint32_t* counts = base + 3ull * kMaxKeys;
    uint32_t* digit_total = counts + 256ull * kMaxBlocks;
    const uint32_t passes = sort_passes(key_bits);
    NA_CUDA(launch_iota(vbuf[0], n, s));
    NA_CUDA(launch_radix_passes(kbuf, vbuf, n, passes, counts, digit_total,
                                false, nullptr, s));
    const int r = passes & 1;
    if (r)
        NA_CUDA(cudaMemcpyAsync(keys, kbuf[1], n * 4ull,
                                cudaMemcpyDeviceToDevice, s));
    if (perm)
        NA_CUDA(cudaMemcpyAsync(perm, vbuf[r], n * 4ull,
                                cudaMemcpyDeviceToDevice, s));
    if (inv_perm)
        NA_CUDA(launch_inverse_perm(vbuf[r], inv_perm, n, nullptr, s));
    return AQUA_OK;
}
