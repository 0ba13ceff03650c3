// aqua_radix_sort_noalloc(): the stable radix sort for callers that must not
// allocate device memory.
//
// Some hosts of this library cannot call cudaMalloc: a tool that runs inside
// another runtime's step loop where every device buffer is owned and sized
// up front by that runtime (as the reference's Variables registry does),
// code running while a stream is being captured into a CUDA graph, or a
// process that works under a fixed device-memory budget.  Such callers get
// a sort that needs no context: its scratch is the file-scope array below.
//
// Limits and sharing:
//   - at most AQUA_NOALLOC_SORT_MAX_KEYS keys per call (larger sizes are
//     rejected with AQUA_ERR_CAPACITY before anything is launched);
//   - all calls in one CUDA context share the one array and it keeps the
//     contents of the last call: calls whose work overlaps on the GPU
//     (different streams without ordering between them) race and give wrong
//     results;
//   - the array belongs to the library's module in a CUDA context, so its
//     device address differs between contexts (a driver-API host's own
//     context, the primary context re-created after cudaDeviceReset).  The
//     address is looked up (cudaGetSymbolAddress) the first time a context
//     calls, and again whenever the calling thread's current context is one
//     not seen before; contexts are told apart by their unique id
//     (cuCtxGetId), never by device index or handle value;
//   - that first call in a context is also where the array's memory is
//     committed (CUDA loads modules lazily), so under a fixed budget it is
//     the call that can fail; make it before any stream capture.  A call
//     that would need the lookup while its stream is capturing returns
//     AQUA_ERR_INVALID without launching anything.
#include <cstdio>
#include <mutex>

#include <cuda.h>

#include "aqua_internal.cuh"
#include "kernels.cuh"

using namespace aqua;

namespace {

constexpr uint32_t kMaxKeys = AQUA_NOALLOC_SORT_MAX_KEYS;
constexpr uint32_t kMaxBlocks = (kMaxKeys + kSortTile - 1) / kSortTile;
// keys ping-pong partner, values ping-pong pair, the sort scratch (digit
// histograms and counters: 1,056 words; two look-back status arrays of 256
// words per tile)
constexpr size_t kSortWords = 4ull * 256ull + 32ull + 2ull * 256ull * kMaxBlocks;
constexpr size_t kWords = 3ull * kMaxKeys + kSortWords;

static __device__ __align__(256) uint32_t g_sort_scratch[kWords];

// Scratch addresses per CUDA context, keyed by the context's unique id
constexpr int kMaxContexts = 32;
struct ScratchEntry
{
    unsigned long long ctx_id;
    uint32_t* ptr;
};
std::mutex g_mutex;
ScratchEntry g_entries[kMaxContexts] = {};
int g_n_entries = 0;
int g_next_victim = 0;

// Driver entry points for the current context and its id, fetched through
// the runtime (the library does not link libcuda directly)
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

bool
driver_entry_points()
{
    if (g_ctx_get_current && g_ctx_get_id)
        return true;
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000,
                                         cudaEnableDefault, &q1) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000,
                                         cudaEnableDefault, &q2) != cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess ||
        !f1 || !f2)
        return false;
    g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
    g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
    return true;
}

// Device address of g_sort_scratch in the calling thread's current context
// (looked up once per context; refused while `stream` is capturing)
aqua_status
scratch_for_current_context(cudaStream_t stream, uint32_t** out)
{
    // binds the device's primary context when no context is current yet
    if (cudaFree(nullptr) != cudaSuccess)
        return AQUA_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!driver_entry_points()) {
        std::fprintf(stderr, "aqua_radix_sort_noalloc: the driver entry points "
                             "cuCtxGetCurrent / cuCtxGetId are unavailable\n");
        return AQUA_ERR_CUDA;
    }
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx ||
        g_ctx_get_id(ctx, &id) != CUDA_SUCCESS)
        return AQUA_ERR_CUDA;
    for (int k = 0; k < g_n_entries; k++)
        if (g_entries[k].ctx_id == id) {
            *out = g_entries[k].ptr;
            return AQUA_OK;
        }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &cap) != cudaSuccess ||
        cap != cudaStreamCaptureStatusNone) {
        std::fprintf(stderr, "aqua_radix_sort_noalloc: the first call in a CUDA "
                             "context must come before any stream capture\n");
        return AQUA_ERR_INVALID;
    }
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_sort_scratch);
    if (e != cudaSuccess || p == nullptr) {
        std::fprintf(stderr, "aqua_radix_sort_noalloc: cudaGetSymbolAddress "
                             "failed: %s\n", cudaGetErrorString(e));
        return AQUA_ERR_CUDA;
    }
    int slot = g_n_entries;
    if (g_n_entries < kMaxContexts) {
        g_n_entries++;
    } else {
        slot = g_next_victim;
        g_next_victim = (g_next_victim + 1) % kMaxContexts;
    }
    g_entries[slot].ctx_id = id;
    g_entries[slot].ptr = static_cast<uint32_t*>(p);
    *out = g_entries[slot].ptr;
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
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint32_t* base = nullptr;
    const aqua_status st = scratch_for_current_context(s, &base);
    if (st != AQUA_OK)
        return st;
    // the caller's keys are one half of the key ping-pong (sorted in place)
    uint32_t* kbuf[2] = { keys, base };
    uint32_t* vbuf[2] = { base + kMaxKeys, base + 2ull * kMaxKeys };
    uint32_t* sort_scratch = base + 3ull * kMaxKeys;
    const uint32_t passes = sort_passes(key_bits);
    if (sort_scratch_words(n) > kSortWords)
        return AQUA_ERR_CAPACITY;
    NA_CUDA(launch_radix_passes(kbuf, vbuf, n, passes, sort_scratch, false,
                                nullptr, s));
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
