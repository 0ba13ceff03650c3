// Link-list of the WCSPH step on sm_103a: bounding box of the positions,
// cell hash, stable LSD radix sort of the cell keys, cell table.
//
// Reference behaviour (paths in the AQUAgpusph tree):
//   r_min / r_max   Reduction tools over r_in, LinkList.cpp:80-91, 338-347
//   n_cells         LinkList::nCells, LinkList.cpp:185-232: per axis
//                   (size_t)((max - min) / (support*h)) + 6, float division
//   icell           iCell, LinkList.cl.in:54-85: (size_t)((r - min) *
//                   (1/(support*h))) + 2 per axis, x fastest
//   sort            RadixSort tool, RadixSort.cpp:130-304 (LSD, stable):
//                   perm[s] = original index, inverse perm[orig] = s
//   ihoc            iHoc + linkList, LinkList.cl.in:32-42, 92-113: first
//                   sorted index of each cell, N if the cell is empty
//
// GB300 design: the bounding box is a warp reduction with atomics per warp
// and case; the cell hash is fused with the histograms of every radix
// digit; the sort uses 8-bit digits (3 passes below 2^24 cells), one kernel
// per pass with decoupled look-back over tiles of 4096 keys ranked stably
// in shared memory and written out as coalesced runs per digit.
#include "aqua_internal.cuh"
#include "kernels.cuh"

namespace aqua {

namespace {

__device__ __forceinline__ void
atomic_min_float(float* addr, float v)
{
    if (v >= 0.f)
        atomicMin((int*)addr, __float_as_int(v));
    else
        atomicMax((unsigned int*)addr, __float_as_uint(v));
}

__device__ __forceinline__ void
atomic_max_float(float* addr, float v)
{
    if (v >= 0.f)
        atomicMax((int*)addr, __float_as_int(v));
    else
        atomicMin((unsigned int*)addr, __float_as_uint(v));
}

// OpenCL min/max (y if y < x)
__device__ __forceinline__ float
cl_min(float x, float y)
{
    return (y < x) ? y : x;
}
__device__ __forceinline__ float
cl_max(float x, float y)
{
    return (x < y) ? y : x;
}

}  // namespace

// Position the link-list sees for particle i of the source set: the Domain
// tool (Domain.cl:48-90) parks non-finite and out-of-box particles at
// domain_max before the link-list runs.
template<int D>
__device__ __forceinline__ void
domain_position(const Consts& c, const float* r, const int32_t* imove,
                uint32_t i, float out[4], bool& removed)
{
    constexpr int VS = Vec<D>::VS;
    float x[4] = { 0.f, 0.f, 0.f, 0.f };
    Vec<D>::load(r, i, x);
    removed = false;
    if (imove == nullptr || imove[i] > -255) {
        bool o = false;
        for (int k = 0; k < D; k++)
            o = o || isnan(x[k]) || isinf(x[k]) || x[k] < c.domain_min[k] ||
                x[k] > c.domain_max[k];
        if (imove != nullptr && o) {
            removed = true;
            for (int k = 0; k < VS; k++)
                x[k] = c.domain_max[k];
        }
    }
    for (int k = 0; k < 4; k++)
        out[k] = x[k];
}

// Resets the per-step scalars of every case and clears the cell table.
__global__ void
k_begin(DevScalars* sc, CaseScalars* cs, uint32_t n_cases, uint2* cells,
        uint2* wall_range, uint8_t* cell_mark, uint32_t ncap, uint32_t N)
{
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    for (uint32_t k = tid; k < n_cases; k += gridDim.x * blockDim.x) {
        for (int d = 0; d < 4; d++) {
            cs[k].r_min[d] = INFINITY;
            cs[k].r_max[d] = -INFINITY;
        }
        cs[k].dt_next = __float_as_uint(INFINITY);
    }
    if (tid == 0) {
        sc->n_chunks = 0;
        sc->chunk_next = 0;
    }
    if (sc->err)
        return;
    for (uint32_t c = tid; c < ncap; c += gridDim.x * blockDim.x) {
        cells[c] = make_uint2(N, N);
        wall_range[c] = make_uint2(0xffffffffu, 0u);
        if (cell_mark)
            cell_mark[c] = 0;
    }
}

// r_min / r_max of every case over its particles.  Cases are contiguous
// runs of particles, so warps are almost always single-case: each lane keeps
// a running box while the warp's tiles stay in one case, and the warp
// reduces its lanes and issues the atomics only when the case changes and
// at the end.
template<int D>
__global__ void __launch_bounds__(256)
k_minmax(Consts c, const float* r, const int32_t* imove, const uint32_t* cid,
         uint32_t N, CaseScalars* cs, DevScalars* sc)
{
    constexpr int VS = Vec<D>::VS;
    __shared__ float s_box[8][2 * VS];
    __shared__ uint32_t s_case[8];
    if (__syncthreads_or(threadIdx.x == 0 && sc->err))
        return;  // one read for the whole block
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    bool bad = false;
    // per-lane running box of the warp's current case wk (warp-uniform);
    // min and max are exact, so the order of accumulation does not matter
    float wmn[VS], wmx[VS];
    uint32_t wk = 0xffffffffu;
    for (int d = 0; d < VS; d++) {
        wmn[d] = INFINITY;
        wmx[d] = -INFINITY;
    }
    auto flush = [&]() {
        if (wk == 0xffffffffu)
            return;
        for (int d = 0; d < VS; d++) {
            for (int o = 16; o > 0; o >>= 1) {
                wmn[d] = cl_min(wmn[d], __shfl_xor_sync(0xffffffffu, wmn[d], o));
                wmx[d] = cl_max(wmx[d], __shfl_xor_sync(0xffffffffu, wmx[d], o));
            }
            if (lane == 0) {
                atomic_min_float(&cs[wk].r_min[d], wmn[d]);
                atomic_max_float(&cs[wk].r_max[d], wmx[d]);
            }
            wmn[d] = INFINITY;
            wmx[d] = -INFINITY;
        }
    };
    // grid-stride over groups of kMinmaxTiles warp-sized tiles (a warp's
    // lanes adjacent); the group's loads are issued before any is used
    constexpr int kMinmaxTiles = 4;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    for (uint32_t base0 = gw * 32 * kMinmaxTiles; base0 < N;
         base0 += warps * 32 * kMinmaxTiles) {
        float xs[kMinmaxTiles][4];
        uint32_t ks[kMinmaxTiles];
#pragma unroll
        for (int u = 0; u < kMinmaxTiles; u++) {
            const uint32_t i = base0 + u * 32 + lane;
            for (int d = 0; d < 4; d++)
                xs[u][d] = 0.f;
            ks[u] = 0xffffffffu;
            if (i < N) {
                bool removed;
                domain_position<D>(c, r, imove, i, xs[u], removed);
                ks[u] = cid ? cid[i] : 0u;
            }
        }
#pragma unroll
        for (int u = 0; u < kMinmaxTiles; u++) {
            const uint32_t i = base0 + u * 32 + lane;
            const bool valid = i < N;
            const float* x = xs[u];
            const uint32_t k = ks[u];
            float mn[VS], mx[VS];
            for (int d = 0; d < VS; d++) {
                const bool ok = valid && isfinite(x[d]);
                if (valid && !isfinite(x[d]))
                    bad = true;
                mn[d] = ok ? x[d] : INFINITY;
                mx[d] = ok ? x[d] : -INFINITY;
            }
            const uint32_t k0 = __shfl_sync(0xffffffffu, k, 0);
            const bool uniform = __all_sync(0xffffffffu, k == k0 || !valid);
            if (uniform) {
                if (k0 != wk) {
                    flush();
                    wk = k0;
                }
                for (int d = 0; d < VS; d++) {
                    wmn[d] = cl_min(wmn[d], mn[d]);
                    wmx[d] = cl_max(wmx[d], mx[d]);
                }
            } else if (valid) {
                for (int d = 0; d < VS; d++) {
                    atomic_min_float(&cs[k].r_min[d], mn[d]);
                    atomic_max_float(&cs[k].r_max[d], mx[d]);
                }
            }
        }
    }
    // the warps' last boxes: one set of atomics per block when the block's
    // warps ended in the same case (the common single-case run), else one
    // per warp
    for (int d = 0; d < VS; d++) {
        for (int o = 16; o > 0; o >>= 1) {
            wmn[d] = cl_min(wmn[d], __shfl_xor_sync(0xffffffffu, wmn[d], o));
            wmx[d] = cl_max(wmx[d], __shfl_xor_sync(0xffffffffu, wmx[d], o));
        }
    }
    if (lane == 0) {
        s_case[warp] = wk;
        for (int d = 0; d < VS; d++) {
            s_box[warp][d] = wmn[d];
            s_box[warp][VS + d] = wmx[d];
        }
    }
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        const uint32_t k = lane < nw ? s_case[lane] : 0xffffffffu;
        const uint32_t k0 = s_case[0];
        const bool same = __all_sync(0xffffffffu, lane >= nw || k == k0);
        for (int d = 0; d < VS; d++) {
            float mn = lane < nw ? s_box[lane][d] : INFINITY;
            float mx = lane < nw ? s_box[lane][VS + d] : -INFINITY;
            if (same) {
                for (int o = 16; o > 0; o >>= 1) {
                    mn = cl_min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
                    mx = cl_max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
                }
                if (lane == 0 && k0 != 0xffffffffu) {
                    atomic_min_float(&cs[k0].r_min[d], mn);
                    atomic_max_float(&cs[k0].r_max[d], mx);
                }
            } else if (lane < nw && k != 0xffffffffu) {
                atomic_min_float(&cs[k].r_min[d], mn);
                atomic_max_float(&cs[k].r_max[d], mx);
            }
        }
    }
    if (__any_sync(0xffffffffu, bad) && lane == 0)
        atomicOr(&sc->err, kErrNonFinite);
}

// n_cells of every case from its bounding box (LinkList::nCells, float
// division), the first global cell key of each case, and the capacity check
template<int D>
__global__ void __launch_bounds__(1024)
k_ncells(Consts c, CaseScalars* cs, uint32_t n_cases, DevScalars* sc,
         uint32_t ncap)
{
    // one block; thread t handles cases [t * per, t * per + per), per <= 4
    __shared__ unsigned long long part[1024];
    __shared__ int bad;
    if (sc->err)
        return;  // the same value for every thread of the block
    if (threadIdx.x == 0)
        bad = 0;
    __syncthreads();
    const uint32_t per = (n_cases + blockDim.x - 1) / blockDim.x;
    const uint32_t k0 = threadIdx.x * per;
    unsigned long long nw[4] = { 0, 0, 0, 0 };
    unsigned long long nn[4][3];
    unsigned long long sum = 0;
    for (uint32_t j = 0; j < per && j < 4; j++) {
        const uint32_t k = k0 + j;
        if (k >= n_cases)
            break;
        nn[j][0] = nn[j][1] = nn[j][2] = 1;
        for (int d = 0; d < D; d++) {
            const float span = (cs[k].r_max[d] - cs[k].r_min[d]) / c.cell_length;
            if (!(span >= 0.f) || span > 4.0e9f)
                bad = 1;
            else
                nn[j][d] = (unsigned long long)span + 6ull;
        }
        nw[j] = nn[j][0] * nn[j][1] * nn[j][2];
        sum += nw[j];
    }
    part[threadIdx.x] = sum;
    __syncthreads();
    for (uint32_t off = 1; off < blockDim.x; off <<= 1) {
        const unsigned long long v = threadIdx.x >= off ? part[threadIdx.x - off] : 0ull;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    const unsigned long long total = part[blockDim.x - 1];
    if (bad || total > ncap) {
        if (threadIdx.x == 0)
            atomicOr(&sc->err, kErrCapacity);
        return;
    }
    unsigned long long base = part[threadIdx.x] - sum;
    for (uint32_t j = 0; j < per && j < 4; j++) {
        const uint32_t k = k0 + j;
        if (k >= n_cases)
            break;
        cs[k].n_cells[0] = (uint32_t)nn[j][0];
        cs[k].n_cells[1] = (uint32_t)nn[j][1];
        cs[k].n_cells[2] = (uint32_t)nn[j][2];
        cs[k].n_cells[3] = (uint32_t)nw[j];
        cs[k].cell_base = (uint32_t)base;
        base += nw[j];
    }
    if (threadIdx.x == 0)
        sc->total_cells = (uint32_t)total;
}

template<int D>
__device__ __forceinline__ uint32_t
cell_of(const Consts& c, const float x[4], const float r_min[4],
        const uint32_t n[4])
{
    uint32_t a[3] = { 0u, 0u, 0u };
    for (int k = 0; k < D; k++)
        a[k] = (uint32_t)(unsigned long long)((x[k] - r_min[k]) * c.idist) + 2u;
    uint32_t cell = a[0] + a[1] * n[0];
    if (D == 3)
        cell += a[2] * n[0] * n[1];
    return cell;
}

// Layout of the sort scratch (sort_scratch_words): the global histogram of
// every digit (kSortMaxPasses x 256), the tile counters of the passes, then
// two look-back status arrays of 256 words per tile that the passes use in
// turn.  A status word holds a count in bits 0-29 and a flag: kStatAgg (the
// tile's own count of the digit) or kStatInc (the count of the digit over
// the tile and every tile before it).
constexpr uint32_t kSortMaxPasses = 4;
constexpr uint32_t kSortHdrWords = kSortMaxPasses * 256 + 32;
constexpr uint32_t kStatAgg = 1u << 30;
constexpr uint32_t kStatInc = 1u << 31;
constexpr uint32_t kStatCount = kStatAgg - 1u;
constexpr uint32_t kLookbackLimit = 1u << 22;
constexpr int kLookbackWindow = 8;

// Adds a key (valid lanes) to the shared histograms of every digit: one
// atomic per run of equal digits over adjacent lanes (the keys of the
// link-list arrive almost sorted, so a warp's lanes form a few runs)
__device__ __forceinline__ void
hist_add_all(uint32_t* hist, uint32_t key, bool valid, uint32_t passes)
{
    const int lane = threadIdx.x & 31;
    for (uint32_t p = 0; p < passes; p++) {
        const uint32_t d = valid ? ((key >> (8 * p)) & 255u) : 256u;
        const uint32_t prev = __shfl_up_sync(0xffffffffu, d, 1);
        const bool head = lane == 0 || prev != d;
        const unsigned heads = __ballot_sync(0xffffffffu, head);
        if (head && valid) {
            const unsigned above = heads & ~((2u << lane) - 1u);
            const int next = above ? __ffs(above) - 1 : 32;
            atomicAdd(&hist[p * 256 + d], (uint32_t)(next - lane));
        }
    }
}

__device__ __forceinline__ void
hist_flush_all(const uint32_t* hist, uint32_t* ghist, uint32_t passes)
{
    for (uint32_t k = threadIdx.x; k < passes * 256; k += blockDim.x)
        if (hist[k])
            atomicAdd(&ghist[k], hist[k]);
}

// icell of every particle (keys: the case's first cell + the local cell)
// and the histograms of every radix digit of the keys, summed into the
// sort scratch
template<int D>
__global__ void __launch_bounds__(kSortThreads)
k_icell_hist(Consts c, const float* r, const int32_t* imove, const uint32_t* cid,
             uint32_t N, const CaseScalars* cs, DevScalars* sc, uint32_t* keys,
             uint32_t* ghist, uint32_t passes)
{
    __shared__ uint32_t hist[kSortMaxPasses * 256];
    for (uint32_t k = threadIdx.x; k < kSortMaxPasses * 256; k += blockDim.x)
        hist[k] = 0;
    if (__syncthreads_or(threadIdx.x == 0 && sc->err))
        return;  // one read for the whole block
    // grid-stride over the keys (a grid of a few blocks per SM keeps the
    // global histogram atomics few)
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < N; i0 += stride) {
        const uint32_t i = i0 + threadIdx.x;
        const bool valid = i < N;
        uint32_t key = 0;
        if (valid) {
            float x[4];
            bool removed;
            domain_position<D>(c, r, imove, i, x, removed);
            const CaseScalars& k = cs[cid ? cid[i] : 0u];
            key = k.cell_base + cell_of<D>(c, x, k.r_min, k.n_cells);
            keys[i] = key;
        }
        hist_add_all(hist, key, valid, passes);
    }
    __syncthreads();
    hist_flush_all(hist, ghist, passes);
}

// Histograms of every radix digit of given keys (the standalone sort)
__global__ void __launch_bounds__(kSortThreads)
k_hist_all(const uint32_t* keys, uint32_t N, uint32_t passes, uint32_t* ghist)
{
    __shared__ uint32_t hist[kSortMaxPasses * 256];
    for (uint32_t k = threadIdx.x; k < kSortMaxPasses * 256; k += blockDim.x)
        hist[k] = 0;
    __syncthreads();
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < N; i0 += stride) {
        const uint32_t i = i0 + threadIdx.x;
        hist_add_all(hist, i < N ? keys[i] : 0u, i < N, passes);
    }
    __syncthreads();
    hist_flush_all(hist, ghist, passes);
}

// Block-wide exclusive scan of one value per thread (256 threads)
__device__ __forceinline__ uint32_t
block_exclusive_scan_256(uint32_t v, uint32_t* s_warp, uint32_t& total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o)
            x += y;
    }
    if (lane == 31)
        s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = (lane < 8) ? s_warp[lane] : 0u;
        for (int o = 1; o < 8; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o)
                w += y;
        }
        if (lane < 8)
            s_warp[lane] = w;  // inclusive warp totals
    }
    __syncthreads();
    total = s_warp[7];
    const uint32_t warp_base = (warp > 0) ? s_warp[warp - 1] : 0u;
    const uint32_t r = warp_base + x - v;
    __syncthreads();
    return r;
}

// Status words are self-contained (count and flag in one 32-bit word, and
// nothing else is read on the strength of a flag), so relaxed accesses at
// GPU scope suffice; they let the loads of a look-back window overlap.
__device__ __forceinline__ uint32_t
ld_status(const uint32_t* p)
{
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void
st_status(uint32_t* p, uint32_t v)
{
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;\n" :: "l"(p), "r"(v) : "memory");
}

// One stable pass of the LSD radix sort over 8-bit digit `shift / 8`, as a
// single kernel with decoupled look-back.  Tiles of kSortTile keys are taken
// in order from an atomic counter (a tile only waits for tiles taken before
// it, whose blocks are running or done).  A tile ranks its keys stably in
// shared memory (per-warp digit counters, ties in index order), publishes
// its per-digit counts, then each thread walks back over the status words
// of its digit until it meets an inclusive count: the exclusive prefix of
// the digit over the previous tiles.  The keys leave as coalesced runs per
// digit.  vals_in == nullptr stands for the identity (the first pass).
// The pass also clears the other status array for the next pass.  A walk
// that finds no status after kLookbackLimit polls records kErrTimeout and
// goes on with what it has.
__global__ void __launch_bounds__(kSortThreads, 3)
k_onesweep(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
           uint32_t* vals_out, uint32_t N, uint32_t shift,
           const uint32_t* ghist, uint32_t* counter, uint32_t* status,
           uint32_t* status_next, DevScalars* sc)
{
    __shared__ uint32_t s_keys[kSortTile];
    __shared__ uint32_t s_vals[kSortTile];
    __shared__ uint32_t s_whist[kSortThreads / 32][256];
    __shared__ uint32_t s_lbase[256];
    __shared__ uint32_t s_gstart[256];
    __shared__ uint32_t s_warp[8];
    __shared__ uint32_t s_tile;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    if (sc != nullptr && sc->err)
        return;  // the same for every block: no tile is taken
    const uint32_t gh = ghist[t];  // the digit's histogram (any tile)
    if (t == 0)
        s_tile = atomicAdd(counter, 1u);
    for (int w = 0; w < kSortThreads / 32; w++)
        s_whist[w][t] = 0;
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t base = tile * kSortTile;

    // the tile's keys and values (warp w holds keys [512 w, 512 w + 512)),
    // in flight during the scan below
    constexpr int kWarpKeys = kSortItems * 32;
    const unsigned lt = (1u << lane) - 1u;
    uint32_t k[kSortItems], v[kSortItems], rk[kSortItems / 2];  // ranks: 16-bit halves
#pragma unroll
    for (int it = 0; it < kSortItems; it++) {
        const uint32_t i = base + warp * kWarpKeys + it * 32 + lane;
        k[it] = (i < N) ? keys_in[i] : 0xffffffffu;
        v[it] = (i < N) ? (vals_in ? vals_in[i] : i) : 0u;
    }
    status_next[(size_t)tile * 256 + t] = 0;

    // the global start of each digit: exclusive scan of its histogram
    uint32_t total;
    const uint32_t gbase = block_exclusive_scan_256(gh, s_warp, total);

    // stable ranks within the tile
#pragma unroll
    for (int it = 0; it < kSortItems; it++) {
        const uint32_t i = base + warp * kWarpKeys + it * 32 + lane;
        const bool valid = i < N;
        const uint32_t d = valid ? ((k[it] >> shift) & 255u) : 256u;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const uint32_t before = valid ? s_whist[warp][d] : 0u;
        __syncwarp();
        if (valid && lane == __ffs(peers) - 1)
            s_whist[warp][d] = before + __popc(peers);
        __syncwarp();
        const uint32_t rank = before + __popc(peers & lt);
        if (it & 1)
            rk[it >> 1] |= rank << 16;
        else
            rk[it >> 1] = rank;
    }
    __syncthreads();
    // thread t = digit t: the warps' offsets, the tile's count
    uint32_t cnt = 0;
    for (int w = 0; w < kSortThreads / 32; w++) {
        const uint32_t c = s_whist[w][t];
        s_whist[w][t] = cnt;
        cnt += c;
    }
    uint32_t tile_total;
    const uint32_t lbase = block_exclusive_scan_256(cnt, s_warp, tile_total);
    s_lbase[t] = lbase;

    // publish, then look back
    uint32_t* st = status + (size_t)tile * 256 + t;
    uint32_t excl = 0;
    if (tile == 0) {
        st_status(st, kStatInc | cnt);
    } else {
        st_status(st, kStatAgg | cnt);
        // the walk reads kLookbackWindow status words at once (tiles
        // p, p - 1, ...; before tile 0 an inclusive zero) and sums them down
        // to the first inclusive one, or up to the first not yet published
        // (then polls again from there)
        int p = (int)tile - 1;
        bool late = true;
        for (uint32_t it = 0; it < kLookbackLimit; it++) {
            uint32_t v[kLookbackWindow];
#pragma unroll
            for (int j = 0; j < kLookbackWindow; j++)
                v[j] = (p - j >= 0) ? ld_status(status + (size_t)(p - j) * 256 + t)
                                    : kStatInc;
            bool done = false;
            int used = 0;  // the leading status words summed
#pragma unroll
            for (int j = 0; j < kLookbackWindow; j++) {
                if (done || used < j || !(v[j] & (kStatAgg | kStatInc)))
                    continue;
                excl += v[j] & kStatCount;
                used = j + 1;
                done = (v[j] & kStatInc) != 0;
            }
            if (done) {
                late = false;
                break;
            }
            if (used == 0)
                __nanosleep(100);  // not published yet: yield the issue slots
            p -= used;
        }
        if (late && sc != nullptr)
            atomicOr(&sc->err, kErrTimeout);
        st_status(st, kStatInc | (excl + cnt));
    }
    s_gstart[t] = gbase + excl - lbase;
    __syncthreads();

    // into shared memory by local position
#pragma unroll
    for (int it = 0; it < kSortItems; it++) {
        const uint32_t i = base + warp * kWarpKeys + it * 32 + lane;
        if (i < N) {
            const uint32_t d = (k[it] >> shift) & 255u;
            const uint32_t pos = s_lbase[d] + s_whist[warp][d] +
                                 ((rk[it >> 1] >> (16 * (it & 1))) & 0xffffu);
            s_keys[pos] = k[it];
            s_vals[pos] = v[it];
        }
    }
    __syncthreads();
    // coalesced write-out: local slot q holds a key of digit d, whose
    // global position is gstart[d] + q
    const uint32_t nvalid = (N > base) ? min((uint32_t)kSortTile, N - base) : 0u;
    for (uint32_t q = t; q < nvalid; q += kSortThreads) {
        const uint32_t key = s_keys[q];
        const uint32_t g = s_gstart[(key >> shift) & 255u] + q;
        keys_out[g] = key;
        vals_out[g] = s_vals[q];
    }
}

// inverse permutation (optional output of the sort tool)
__global__ void
k_inverse_perm(const uint32_t* perm, uint32_t* inv, uint32_t n,
               const DevScalars* sc)
{
    if (sc != nullptr && sc->err)
        return;
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n)
        inv[perm[s]] = s;
}

// cell table of sorted keys (standalone link-list): ihoc[c] = first index
__global__ void
k_ihoc(const uint32_t* keys, uint32_t n, uint32_t* ihoc, const DevScalars* sc)
{
    if (sc != nullptr && sc->err)
        return;
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n)
        return;
    const uint32_t k = keys[s];
    if (s == 0 || keys[s - 1] != k)
        ihoc[k] = s;
}

__global__ void
k_iota(uint32_t* p, uint32_t n)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        p[i] = i;
}

__global__ void
k_fill_u32(uint32_t* p, uint32_t v, uint32_t n, const DevScalars* sc)
{
    if (sc != nullptr && sc->err)
        return;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x)
        p[i] = v;
}

// --------------------------------------------------------------- launchers

static inline unsigned
grid_for(uint32_t n, unsigned threads)
{
    return (unsigned)((n + threads - 1) / threads);
}

cudaError_t
launch_begin(DevScalars* sc, CaseScalars* cs, uint32_t n_cases, uint2* cells,
             uint2* wall_range, uint8_t* cell_mark, uint32_t ncap, uint32_t N,
             cudaStream_t s)
{
    const unsigned g = min(grid_for(max(ncap, n_cases), 256), 152u * 8u);
    k_begin<<<max(g, 1u), 256, 0, s>>>(sc, cs, n_cases, cells, wall_range,
                                        cell_mark, ncap, N);
    return cudaGetLastError();
}

template<int D>
cudaError_t
launch_minmax(const Consts& c, const float* r, const int32_t* imove,
              const uint32_t* cid, uint32_t N, CaseScalars* cs, DevScalars* sc,
              cudaStream_t s)
{
    const unsigned g = min(grid_for(N, 256), 152u * 4u);
    k_minmax<D><<<max(g, 1u), 256, 0, s>>>(c, r, imove, cid, N, cs, sc);
    return cudaGetLastError();
}

template<int D>
cudaError_t
launch_ncells(const Consts& c, CaseScalars* cs, uint32_t n_cases, DevScalars* sc,
              uint32_t ncap, cudaStream_t s)
{
    k_ncells<D><<<1, 1024, 0, s>>>(c, cs, n_cases, sc, ncap);
    return cudaGetLastError();
}

uint32_t
sort_blocks(uint32_t n)
{
    return (n + kSortTile - 1) / kSortTile;
}

uint32_t
sort_passes(uint32_t key_bits)
{
    return key_bits == 0 ? 1u : (key_bits + 7u) / 8u;
}

// blocks of the histogram kernels: at most 4 per SM
static inline unsigned
hist_grid(uint32_t n)
{
    return max(1u, min(grid_for(n, kSortThreads), 152u * 4u));
}

size_t
sort_scratch_words(uint32_t n)
{
    return kSortHdrWords + 2ull * 256ull * sort_blocks(n);
}

// Clears the histograms, the tile counters and the first pass's status
// array of the sort scratch (before the histograms are summed)
cudaError_t
launch_sort_reset(uint32_t* scratch, uint32_t n, cudaStream_t s)
{
    const size_t words = kSortHdrWords + 256ull * sort_blocks(n);
    return cudaMemsetAsync(scratch, 0, words * 4ull, s);
}

// Radix passes on the keys in keys[0] (values: the identity); the result
// lands in keys/vals[passes & 1].  The scratch is reset here unless
// `hist_ready` (the caller reset it and summed the histograms).
cudaError_t
launch_radix_passes(uint32_t* keys[2], uint32_t* vals[2], uint32_t n,
                    uint32_t passes, uint32_t* scratch, bool hist_ready,
                    DevScalars* sc, cudaStream_t s)
{
    const uint32_t nb = sort_blocks(n);
    if (nb == 0)
        return cudaSuccess;
    if (passes > kSortMaxPasses || n >= kStatAgg)
        return cudaErrorInvalidValue;
    uint32_t* ghist = scratch;
    uint32_t* counters = scratch + kSortMaxPasses * 256;
    uint32_t* stat[2] = { scratch + kSortHdrWords,
                          scratch + kSortHdrWords + 256ull * nb };
    if (!hist_ready) {
        cudaError_t e = launch_sort_reset(scratch, n, s);
        if (e != cudaSuccess)
            return e;
        k_hist_all<<<hist_grid(n), kSortThreads, 0, s>>>(keys[0], n, passes,
                                                         ghist);
    }
    for (uint32_t p = 0; p < passes; p++) {
        const int in = p & 1, out = in ^ 1;
        k_onesweep<<<nb, kSortThreads, 0, s>>>(
            keys[in], p == 0 ? nullptr : vals[in], keys[out], vals[out], n,
            8u * p, ghist + 256 * p, counters + p, stat[p & 1],
            stat[(p + 1) & 1], sc);
    }
    return cudaGetLastError();
}

template<int D>
cudaError_t
launch_icell_hist(const Consts& c, const float* r, const int32_t* imove,
                  const uint32_t* cid, uint32_t N, const CaseScalars* cs,
                  DevScalars* sc, uint32_t* keys, uint32_t* scratch,
                  uint32_t passes, cudaStream_t s)
{
    const uint32_t nb = sort_blocks(N);
    if (nb == 0)
        return cudaSuccess;
    cudaError_t e = launch_sort_reset(scratch, N, s);
    if (e != cudaSuccess)
        return e;
    k_icell_hist<D><<<hist_grid(N), kSortThreads, 0, s>>>(
        c, r, imove, cid, N, cs, sc, keys, scratch, passes);
    return cudaGetLastError();
}

cudaError_t
launch_inverse_perm(const uint32_t* perm, uint32_t* inv, uint32_t n,
                    const DevScalars* sc, cudaStream_t s)
{
    if (n == 0)
        return cudaSuccess;
    k_inverse_perm<<<grid_for(n, 256), 256, 0, s>>>(perm, inv, n, sc);
    return cudaGetLastError();
}

cudaError_t
launch_ihoc(const uint32_t* keys, uint32_t n, uint32_t* ihoc, uint32_t ncap,
            const DevScalars* sc, cudaStream_t s)
{
    const unsigned g = min(grid_for(ncap, 256), 152u * 8u);
    k_fill_u32<<<max(g, 1u), 256, 0, s>>>(ihoc, n, ncap, sc);
    if (n)
        k_ihoc<<<grid_for(n, 256), 256, 0, s>>>(keys, n, ihoc, sc);
    return cudaGetLastError();
}

cudaError_t
launch_iota(uint32_t* p, uint32_t n, cudaStream_t s)
{
    if (n)
        k_iota<<<grid_for(n, 256), 256, 0, s>>>(p, n);
    return cudaGetLastError();
}

template cudaError_t launch_minmax<2>(const Consts&, const float*,
                                      const int32_t*, const uint32_t*, uint32_t,
                                      CaseScalars*, DevScalars*, cudaStream_t);
template cudaError_t launch_minmax<3>(const Consts&, const float*,
                                      const int32_t*, const uint32_t*, uint32_t,
                                      CaseScalars*, DevScalars*, cudaStream_t);
template cudaError_t launch_ncells<2>(const Consts&, CaseScalars*, uint32_t,
                                      DevScalars*, uint32_t, cudaStream_t);
template cudaError_t launch_ncells<3>(const Consts&, CaseScalars*, uint32_t,
                                      DevScalars*, uint32_t, cudaStream_t);
template cudaError_t launch_icell_hist<2>(const Consts&, const float*,
                                          const int32_t*, const uint32_t*,
                                          uint32_t, const CaseScalars*,
                                          DevScalars*, uint32_t*, uint32_t*,
                                          uint32_t, cudaStream_t);
template cudaError_t launch_icell_hist<3>(const Consts&, const float*,
                                          const int32_t*, const uint32_t*,
                                          uint32_t, const CaseScalars*,
                                          DevScalars*, uint32_t*, uint32_t*,
                                          uint32_t, cudaStream_t);

}  // namespace aqua
