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
// GB300 design: the bounding box is a block reduction with one float
// atomic per block; the cell hash is fused with the first radix pass's
// histogram; the sort uses 8-bit digits (3 passes below 2^24 cells) with
// per-block tiles of 4096 keys ranked stably in shared memory and written
// out as coalesced runs per digit.
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
        sc->n_clusters = 0;
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
    if (sc->err)
        return;
    const int lane = threadIdx.x & 31;
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
    // grid-stride over warp-sized tiles so that a warp's lanes are adjacent
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    for (uint32_t base = gw * 32; base < N; base += warps * 32) {
        const uint32_t i = base + lane;
        const bool valid = i < N;
        float x[4] = { 0.f, 0.f, 0.f, 0.f };
        uint32_t k = 0xffffffffu;
        if (valid) {
            bool removed;
            domain_position<D>(c, r, imove, i, x, removed);
            k = cid ? cid[i] : 0u;
        }
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
    flush();
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

// icell of every particle (keys: the case's first cell + the local cell),
// identity values, and the histogram of the first radix digit per tile
template<int D>
__global__ void __launch_bounds__(kSortThreads)
k_icell_hist(Consts c, const float* r, const int32_t* imove, const uint32_t* cid,
             uint32_t N, const CaseScalars* cs, DevScalars* sc, uint32_t* keys,
             uint32_t* vals, uint32_t* counts, uint32_t nblocks)
{
    __shared__ uint32_t hist[256];
    hist[threadIdx.x] = 0;
    __syncthreads();
    if (sc->err)
        return;
    const uint32_t base = blockIdx.x * kSortTile;
    for (int it = 0; it < kSortItems; it++) {
        const uint32_t i = base + it * kSortThreads + threadIdx.x;
        if (i >= N)
            break;
        float x[4];
        bool removed;
        domain_position<D>(c, r, imove, i, x, removed);
        const CaseScalars& k = cs[cid ? cid[i] : 0u];
        const uint32_t key = k.cell_base + cell_of<D>(c, x, k.r_min, k.n_cells);
        keys[i] = key;
        vals[i] = i;
        atomicAdd(&hist[key & 255u], 1u);
    }
    __syncthreads();
    counts[threadIdx.x * nblocks + blockIdx.x] = hist[threadIdx.x];
}

// Histogram of one radix digit per tile
__global__ void __launch_bounds__(kSortThreads)
k_hist(const uint32_t* keys, uint32_t N, uint32_t shift, uint32_t* counts,
       uint32_t nblocks, const DevScalars* sc)
{
    __shared__ uint32_t hist[256];
    hist[threadIdx.x] = 0;
    __syncthreads();
    if (sc != nullptr && sc->err)
        return;
    const uint32_t base = blockIdx.x * kSortTile;
    for (int it = 0; it < kSortItems; it++) {
        const uint32_t i = base + it * kSortThreads + threadIdx.x;
        if (i >= N)
            break;
        atomicAdd(&hist[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    counts[threadIdx.x * nblocks + blockIdx.x] = hist[threadIdx.x];
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

// One block per digit: exclusive scan of the digit's per-tile counts, and
// the digit total
__global__ void __launch_bounds__(kSortThreads)
k_scan_rows(uint32_t* counts, uint32_t nblocks, uint32_t* digit_total,
            const DevScalars* sc)
{
    __shared__ uint32_t s_warp[8];
    if (sc != nullptr && sc->err)
        return;
    uint32_t* row = counts + (size_t)blockIdx.x * nblocks;
    const uint32_t per = (nblocks + kSortThreads - 1) / kSortThreads;
    const uint32_t b0 = threadIdx.x * per;
    uint32_t sum = 0;
    for (uint32_t k = 0; k < per; k++) {
        const uint32_t b = b0 + k;
        if (b < nblocks)
            sum += row[b];
    }
    uint32_t total;
    uint32_t run = block_exclusive_scan_256(sum, s_warp, total);
    for (uint32_t k = 0; k < per; k++) {
        const uint32_t b = b0 + k;
        if (b < nblocks) {
            const uint32_t v = row[b];
            row[b] = run;
            run += v;
        }
    }
    if (threadIdx.x == 0)
        digit_total[blockIdx.x] = total;
}

// Stable scatter of one radix digit: rank the tile's keys by digit in
// shared memory (ties in index order), then write coalesced runs.
__global__ void __launch_bounds__(kSortThreads)
k_scatter(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
          uint32_t* vals_out, uint32_t N, uint32_t shift,
          const uint32_t* counts, uint32_t nblocks,
          const uint32_t* digit_total, const DevScalars* sc)
{
    __shared__ uint32_t s_keys[kSortTile];
    __shared__ uint32_t s_vals[kSortTile];
    __shared__ uint32_t s_wcnt[kSortThreads / 32][256];
    __shared__ uint32_t s_local[256];   // running local offset per digit
    __shared__ uint32_t s_lbase[256];   // local start of each digit
    __shared__ uint32_t s_gbase[256];   // global start of each digit
    __shared__ uint32_t s_warp[8];
    if (sc != nullptr && sc->err)
        return;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t base = blockIdx.x * kSortTile;

    // keys of this tile in registers; per-digit counts of the tile
    uint32_t k[kSortItems];
    for (int w = 0; w < kSortThreads / 32; w++)
        s_wcnt[w][t] = 0;
    s_local[t] = 0;
    __syncthreads();
    for (int it = 0; it < kSortItems; it++) {
        const uint32_t i = base + it * kSortThreads + t;
        k[it] = (i < N) ? keys_in[i] : 0xffffffffu;
        if (i < N)
            atomicAdd(&s_local[(k[it] >> shift) & 255u], 1u);
    }
    __syncthreads();
    {
        uint32_t total;
        const uint32_t cnt = s_local[t];
        const uint32_t ex = block_exclusive_scan_256(cnt, s_warp, total);
        s_lbase[t] = ex;
        s_local[t] = ex;
        // global base of the digit: exclusive scan of the digit totals
        const uint32_t dt = digit_total[t];
        uint32_t total2;
        const uint32_t gex = block_exclusive_scan_256(dt, s_warp, total2);
        s_gbase[t] = gex + counts[(size_t)t * nblocks + blockIdx.x];
    }
    __syncthreads();

    const unsigned lt_mask = (1u << lane) - 1u;
    for (int it = 0; it < kSortItems; it++) {
        const uint32_t i = base + it * kSortThreads + t;
        const bool valid = i < N;
        const uint32_t d = valid ? ((k[it] >> shift) & 255u) : 256u;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const uint32_t rank = __popc(peers & lt_mask);
        if (valid && rank == 0)
            s_wcnt[warp][d] = __popc(peers);
        __syncthreads();
        {
            uint32_t run = s_local[t];
            for (int w = 0; w < kSortThreads / 32; w++) {
                const uint32_t cnum = s_wcnt[w][t];
                s_wcnt[w][t] = run;
                run += cnum;
            }
            s_local[t] = run;
        }
        __syncthreads();
        if (valid) {
            const uint32_t pos = s_wcnt[warp][d] + rank;
            s_keys[pos] = k[it];
            s_vals[pos] = vals_in[i];
        }
        __syncthreads();
        for (int w = 0; w < kSortThreads / 32; w++)
            s_wcnt[w][t] = 0;
        __syncthreads();
    }
    // coalesced write-out: local slot p holds a key of digit d, whose
    // global position is gbase[d] + (p - lbase[d])
    const uint32_t nvalid = (N > base) ? min((uint32_t)kSortTile, N - base) : 0u;
    for (uint32_t p = t; p < nvalid; p += kSortThreads) {
        const uint32_t key = s_keys[p];
        const uint32_t d = (key >> shift) & 255u;
        const uint32_t g = s_gbase[d] + (p - s_lbase[d]);
        keys_out[g] = key;
        vals_out[g] = s_vals[p];
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

// Radix passes on keys/vals already in bufs[0] (pass-0 counts ready if
// `first_counts_ready`); result lands in bufs[passes & 1].
cudaError_t
launch_radix_passes(uint32_t* keys[2], uint32_t* vals[2], uint32_t n,
                    uint32_t passes, uint32_t* counts, uint32_t* digit_total,
                    bool first_counts_ready, const DevScalars* sc,
                    cudaStream_t s)
{
    const uint32_t nb = sort_blocks(n);
    if (nb == 0)
        return cudaSuccess;
    for (uint32_t p = 0; p < passes; p++) {
        const uint32_t shift = 8u * p;
        const int in = p & 1, out = in ^ 1;
        if (p > 0 || !first_counts_ready)
            k_hist<<<nb, kSortThreads, 0, s>>>(keys[in], n, shift, counts, nb, sc);
        k_scan_rows<<<256, kSortThreads, 0, s>>>(counts, nb, digit_total, sc);
        k_scatter<<<nb, kSortThreads, 0, s>>>(keys[in], vals[in], keys[out],
                                              vals[out], n, shift, counts, nb,
                                              digit_total, sc);
    }
    return cudaGetLastError();
}

template<int D>
cudaError_t
launch_icell_hist(const Consts& c, const float* r, const int32_t* imove,
                  const uint32_t* cid, uint32_t N, const CaseScalars* cs,
                  DevScalars* sc, uint32_t* keys, uint32_t* vals,
                  uint32_t* counts, cudaStream_t s)
{
    const uint32_t nb = sort_blocks(N);
    if (nb == 0)
        return cudaSuccess;
    k_icell_hist<D><<<nb, kSortThreads, 0, s>>>(c, r, imove, cid, N, cs, sc,
                                                 keys, vals, counts, nb);
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
                                          uint32_t*, cudaStream_t);
template cudaError_t launch_icell_hist<3>(const Consts&, const float*,
                                          const int32_t*, const uint32_t*,
                                          uint32_t, const CaseScalars*,
                                          DevScalars*, uint32_t*, uint32_t*,
                                          uint32_t*, cudaStream_t);

}  // namespace aqua
