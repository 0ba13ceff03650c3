// Kernels of the learned k-step proposal (include/aqua_learned.h): the
// neighbour graph, node / edge features, dense layers on the tensor cores
// (BF16 x BF16 -> FP32, mma.sync m16n8k16), graph aggregation, loss, Adam
// and the application of a proposal to the particle state.  No counterpart
// in the reference.
#include <cuda_bf16.h>
#include <cstdint>

#include "aqua_learned.h"
#include "aqua_internal.cuh"  // sample_hash: the cells of a rate sample

namespace {

using bf16 = __nv_bfloat16;

#define GNN_CUDA(call)                                                         \
    do {                                                                       \
        if ((call) != cudaSuccess)                                             \
            return AQUA_ERR_CUDA;                                              \
    } while (0)

inline aqua_status
last_error()
{
    return cudaGetLastError() == cudaSuccess ? AQUA_OK : AQUA_ERR_CUDA;
}

inline unsigned
blocks_for(uint64_t n, unsigned threads, unsigned cap = 65535u * 4u)
{
    const uint64_t b = (n + threads - 1) / threads;
    return b == 0 ? 1u : (b > cap ? cap : (unsigned)b);
}

__device__ __forceinline__ float
bf2f(uint16_t v)
{
    return __uint_as_float((uint32_t)v << 16);
}

__device__ __forceinline__ uint16_t
f2bf(float f)
{
    return __bfloat16_as_ushort(__float2bfloat16_rn(f));
}

__device__ __forceinline__ uint32_t
pack_bf2(float lo, float hi)
{
    return (uint32_t)f2bf(lo) | ((uint32_t)f2bf(hi) << 16);
}

__device__ __forceinline__ float
sigmoid(float z)
{
    return 1.f / (1.f + expf(-z));
}

__device__ __forceinline__ float
silu(float z)
{
    return z * sigmoid(z);
}

__device__ __forceinline__ float
silu_grad(float z)
{
    const float s = sigmoid(z);
    return s * (1.f + z * (1.f - s));
}

// D (16x8 f32) += A (16x16 bf16, row) * B (16x8 bf16, col)
__device__ __forceinline__ void
mma_bf16(float c[4], const uint32_t a[4], const uint32_t b[2])
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ void
ldsm_x4_trans(uint32_t r[4], const void* p)
{
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 "
                 "{%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

__device__ __forceinline__ uint32_t
ld_u32(const uint16_t* p)
{
    return *reinterpret_cast<const uint32_t*>(p);
}

// ---------------------------------------------------------------- graph ----

__global__ void
k_cell_keys(uint32_t n, int dims, const float* __restrict__ r,
            const int32_t* __restrict__ imove, const uint32_t* __restrict__ cid,
            float cell, float o0, float o1, float o2, uint32_t n0, uint32_t n1,
            uint32_t n2, uint32_t* keys, uint32_t* vals)
{
    const uint32_t VS = dims == 3 ? 4 : 2;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        vals[i] = i;
        if (imove[i] == 0) {
            keys[i] = 0xffffffffu;
            continue;
        }
        const float o[3] = { o0, o1, o2 };
        const uint32_t nc[3] = { n0, n1, n2 };
        uint32_t c[3] = { 0, 0, 0 };
        for (int d = 0; d < dims; d++) {
            const float x = (r[(size_t)i * VS + d] - o[d]) / cell;
            uint32_t v = 0;
            if (x >= (float)nc[d])
                v = nc[d] - 1;
            else if (x > 0.f)
                v = (uint32_t)x;   // NaN and negatives stay in cell 0
            c[d] = v;
        }
        const uint32_t per_case = n0 * n1 * (dims == 3 ? n2 : 1u);
        keys[i] = cid[i] * per_case + c[0] + n0 * (c[1] + n1 * c[2]);
    }
}

__global__ void
k_fill_u32(uint32_t n, uint32_t v, uint32_t* p)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x)
        p[i] = v;
}

__global__ void
k_cell_ranges(uint32_t n, const uint32_t* __restrict__ k, uint32_t n_keys,
              uint32_t* start, uint32_t* end)
{
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n;
         s += gridDim.x * blockDim.x) {
        const uint32_t key = k[s];
        if (key >= n_keys)
            continue;
        if (s == 0 || k[s - 1] != key)
            start[key] = s;
        if (s + 1 == n || k[s + 1] != key)
            end[key] = s + 1;
    }
}

template<int D>
__global__ void
k_neighbours(uint32_t n, const float* __restrict__ rs,
             const uint32_t* __restrict__ keys, uint32_t n0, uint32_t n1,
             uint32_t n2, const uint32_t* __restrict__ cstart,
             const uint32_t* __restrict__ cend, float r2max, uint32_t* degree,
             const uint32_t* __restrict__ offsets, uint32_t* recv,
             uint32_t* send)
{
    constexpr int VS = D == 3 ? 4 : 2;
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n;
         s += gridDim.x * blockDim.x) {
        const uint32_t key = keys[s];
        const uint32_t per_case = n0 * n1 * (D == 3 ? n2 : 1u);
        const uint32_t base = (key / per_case) * per_case;
        const uint32_t local = key - base;
        const int cx = (int)(local % n0);
        const int cy = (int)((local / n0) % n1);
        const int cz = D == 3 ? (int)(local / (n0 * n1)) : 0;
        float ri[3] = { rs[(size_t)s * VS], rs[(size_t)s * VS + 1],
                        D == 3 ? rs[(size_t)s * VS + 2] : 0.f };
        uint32_t cnt = 0;
        const uint32_t o = send ? offsets[s] : 0u;
        for (int dx = -1; dx <= 1; dx++) {
            const int x = cx + dx;
            if (x < 0 || x >= (int)n0)
                continue;
            for (int dy = -1; dy <= 1; dy++) {
                const int y = cy + dy;
                if (y < 0 || y >= (int)n1)
                    continue;
                for (int dz = (D == 3 ? -1 : 0); dz <= (D == 3 ? 1 : 0); dz++) {
                    const int z = cz + dz;
                    if (D == 3 && (z < 0 || z >= (int)n2))
                        continue;
                    const uint32_t c = base + (uint32_t)x +
                                       n0 * ((uint32_t)y + n1 * (uint32_t)z);
                    const uint32_t b = cstart[c], e = cend[c];
                    for (uint32_t j = b; j < e; j++) {
                        if (j == s)
                            continue;
                        float rr = 0.f;
                        for (int d = 0; d < D; d++) {
                            const float dd = rs[(size_t)j * VS + d] - ri[d];
                            rr += dd * dd;
                        }
                        if (rr < r2max) {
                            if (send) {
                                recv[o + cnt] = s;
                                send[o + cnt] = j;
                            }
                            cnt++;
                        }
                    }
                }
            }
        }
        if (!send)
            degree[s] = cnt;
    }
}

__device__ __forceinline__ int
ordered(float f)
{
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}

__device__ __forceinline__ float
unordered(int i)
{
    return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff);
}

__global__ void
k_bbox_init(int* s)
{
    if (threadIdx.x < 3) {
        s[threadIdx.x] = ordered(INFINITY);
        s[3 + threadIdx.x] = ordered(-INFINITY);
    }
}

__global__ void
k_bbox(uint32_t n, int dims, const float* __restrict__ r,
       const int32_t* __restrict__ imove, int* s)
{
    const uint32_t VS = dims == 3 ? 4 : 2;
    float lo[3] = { INFINITY, INFINITY, INFINITY };
    float hi[3] = { -INFINITY, -INFINITY, -INFINITY };
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        if (imove[i] == 0)
            continue;
        for (int d = 0; d < dims; d++) {
            const float x = r[(size_t)i * VS + d];
            lo[d] = fminf(lo[d], x);
            hi[d] = fmaxf(hi[d], x);
        }
    }
    for (int d = 0; d < 3; d++) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[d] = fminf(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
            hi[d] = fmaxf(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
        }
        if ((threadIdx.x & 31) == 0) {
            if (lo[d] < INFINITY)
                atomicMin(&s[d], ordered(lo[d]));
            if (hi[d] > -INFINITY)
                atomicMax(&s[3 + d], ordered(hi[d]));
        }
    }
}

__global__ void
k_bbox_decode(const int* s, float* out)
{
    if (threadIdx.x < 6)
        out[threadIdx.x] = unordered(s[threadIdx.x]);
}

// exclusive scan, 1024 threads x 4 items per block
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ uint32_t
block_scan_exclusive(uint32_t v, uint32_t* warp_sums, uint32_t* total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o)
            x += y;
    }
    if (lane == 31)
        warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o)
                w += y;
        }
        warp_sums[lane] = w;
    }
    __syncthreads();
    const uint32_t before = warp > 0 ? warp_sums[warp - 1] : 0u;
    if (total)
        *total = warp_sums[(blockDim.x >> 5) - 1];
    return before + x - v;
}

__global__ void __launch_bounds__(kScanThreads)
k_scan_tiles(uint32_t n, const uint32_t* __restrict__ in, uint32_t* out,
             uint32_t* tile_sums)
{
    __shared__ uint32_t ws[32];
    __shared__ uint32_t tot;
    const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t v[kScanItems], s = 0;
    for (int k = 0; k < kScanItems; k++) {
        v[k] = base + k < n ? in[base + k] : 0u;
        s += v[k];
    }
    uint32_t pre = block_scan_exclusive(s, ws, &tot);
    for (int k = 0; k < kScanItems; k++) {
        if (base + k < n)
            out[base + k] = pre;
        pre += v[k];
    }
    if (threadIdx.x == 0)
        tile_sums[blockIdx.x] = tot;
}

// one block: exclusive scan of up to kScanThreads * 16 tile sums in place
__global__ void __launch_bounds__(kScanThreads)
k_scan_sums(uint32_t m, uint32_t* sums, uint32_t* grand)
{
    __shared__ uint32_t ws[32];
    __shared__ uint32_t tot;
    constexpr int P = 16;
    const uint32_t base = threadIdx.x * P;
    uint32_t v[P], s = 0;
    for (int k = 0; k < P; k++) {
        v[k] = base + k < m ? sums[base + k] : 0u;
        s += v[k];
    }
    uint32_t pre = block_scan_exclusive(s, ws, &tot);
    for (int k = 0; k < P; k++) {
        if (base + k < m)
            sums[base + k] = pre;
        pre += v[k];
    }
    if (threadIdx.x == 0)
        *grand = tot;
}

__global__ void
k_scan_add(uint32_t n, uint32_t* out, const uint32_t* __restrict__ sums,
           const uint32_t* grand)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= n;
         i += gridDim.x * blockDim.x) {
        if (i == n)
            out[n] = *grand;
        else
            out[i] += sums[i / kScanTile];
    }
}

__global__ void
k_gather32(uint32_t n, const uint32_t* __restrict__ perm,
           const uint32_t* __restrict__ src, uint32_t stride, uint32_t comps,
           uint32_t* dst)
{
    const uint64_t total = (uint64_t)n * comps;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
         t < total; t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t s = t / comps, c = t % comps;
        dst[t] = src[(uint64_t)perm[s] * stride + c];
    }
}

__global__ void
k_scatter32(uint32_t n, const uint32_t* __restrict__ perm,
            const uint32_t* __restrict__ src, uint32_t comps, uint32_t* dst,
            uint32_t stride)
{
    const uint64_t total = (uint64_t)n * comps;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
         t < total; t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t s = t / comps, c = t % comps;
        dst[(uint64_t)perm[s] * stride + c] = src[t];
    }
}

// ------------------------------------------------------------- features ----

// Wendland C2 shape (1 + 2q)(1 - q/2)^4, q = r / h in [0, 2]; 1 at q = 0
__device__ __forceinline__ float
wendland_shape(float q)
{
    if (!(q < 2.f))
        return 0.f;
    const float a = 1.f - 0.5f * q;
    const float a2 = a * a;
    return (1.f + 2.f * q) * a2 * a2;
}

__global__ void
k_node_features(uint32_t n, int dims, const float* __restrict__ u,
                const float* __restrict__ rho, const float* __restrict__ dudt,
                const float* __restrict__ drhodt,
                const int32_t* __restrict__ imove,
                const float* __restrict__ normal, const float* __restrict__ sc,
                uint16_t* out, uint32_t ld, uint32_t col)
{
    const uint32_t VS = dims == 3 ? 4 : 2;
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n;
         s += gridDim.x * blockDim.x) {
        float f[AQUA_GNN_FEATURES];
        for (int k = 0; k < AQUA_GNN_FEATURES; k++)
            f[k] = 0.f;
        const float U = sc[1], R = sc[2], A = sc[3], Rd = sc[4], rho0 = sc[5];
        const bool fluid = imove[s] == 1, wall = imove[s] < 0;
        int k = 0;
        for (int d = 0; d < dims; d++)
            f[k++] = u[(size_t)s * VS + d] / U;
        f[k++] = (rho[s] - rho0) / R;
        for (int d = 0; d < dims; d++)
            f[k++] = dudt[(size_t)s * VS + d] / A;
        f[k++] = drhodt[s] / Rd;
        f[k++] = fluid ? 1.f : 0.f;
        f[k++] = wall ? 1.f : 0.f;
        for (int d = 0; d < dims; d++)
            f[k++] = wall ? normal[(size_t)s * VS + d] : 0.f;
        uint16_t* row = out + (size_t)s * ld + col;
        for (int j = 0; j < AQUA_GNN_FEATURES; j += 2)
            *reinterpret_cast<uint32_t*>(row + j) = pack_bf2(f[j], f[j + 1]);
    }
}

__global__ void
k_edge_features(uint32_t E, int dims, const uint32_t* __restrict__ recv,
                const uint32_t* __restrict__ send, const float* __restrict__ r,
                const float* __restrict__ u, const float* __restrict__ rho,
                const int32_t* __restrict__ imove,
                const float* __restrict__ normal, const float* __restrict__ sc,
                uint16_t* out)
{
    const uint32_t VS = dims == 3 ? 4 : 2;
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < E;
         e += gridDim.x * blockDim.x) {
        const uint32_t i = recv[e], j = send[e];
        float f[AQUA_GNN_FEATURES];
        for (int k = 0; k < AQUA_GNN_FEATURES; k++)
            f[k] = 0.f;
        const float h = sc[0], U = sc[1], R = sc[2];
        int k = 0;
        float rr = 0.f;
        for (int d = 0; d < dims; d++) {
            const float dd = r[(size_t)j * VS + d] - r[(size_t)i * VS + d];
            rr += dd * dd;
            f[k++] = dd / h;
        }
        const float q = sqrtf(rr) / h;
        f[k++] = q;
        for (int d = 0; d < dims; d++)
            f[k++] = (u[(size_t)j * VS + d] - u[(size_t)i * VS + d]) / U;
        f[k++] = (rho[j] - rho[i]) / R;
        f[k++] = wendland_shape(q);
        const bool wall = imove[j] < 0;
        f[k++] = wall ? 1.f : 0.f;
        for (int d = 0; d < dims; d++)
            f[k++] = wall ? normal[(size_t)j * VS + d] : 0.f;
        uint16_t* row = out + (size_t)e * AQUA_GNN_FEATURES;
        for (int m = 0; m < AQUA_GNN_FEATURES; m += 2)
            *reinterpret_cast<uint32_t*>(row + m) = pack_bf2(f[m], f[m + 1]);
    }
}

// The node data the edge features read, packed per node into 16-byte
// aligned records (2-D: 2 float4 = r, u | rho, imove bits, normal; 3-D:
// 3 float4 = r, rho | u, imove bits | normal, 0), so that an edge reads two
// or three aligned 16-byte words per end instead of ten scattered fields.
template<int D>
__global__ void
k_node_records(uint32_t n, const float* __restrict__ r,
               const float* __restrict__ u, const float* __restrict__ rho,
               const int32_t* __restrict__ imove,
               const float* __restrict__ normal, float4* rec)
{
    constexpr int VS = D == 3 ? 4 : 2;
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n;
         s += gridDim.x * blockDim.x) {
        const float* rs = r + (size_t)s * VS;
        const float* us = u + (size_t)s * VS;
        const float* ns = normal + (size_t)s * VS;
        const float im = __int_as_float(imove[s]);
        if (D == 2) {
            rec[(size_t)s * 2] = make_float4(rs[0], rs[1], us[0], us[1]);
            rec[(size_t)s * 2 + 1] = make_float4(rho[s], im, ns[0], ns[1]);
        } else {
            rec[(size_t)s * 3] = make_float4(rs[0], rs[1], rs[2], rho[s]);
            rec[(size_t)s * 3 + 1] = make_float4(us[0], us[1], us[2], im);
            rec[(size_t)s * 3 + 2] = make_float4(ns[0], ns[1], ns[2], 0.f);
        }
    }
}

// k_edge_features from the packed records: the same features, computed by
// the same operations in the same order
template<int D>
__global__ void
k_edge_features_rec(uint32_t E, const uint32_t* __restrict__ recv,
                    const uint32_t* __restrict__ send,
                    const float4* __restrict__ rec,
                    const float* __restrict__ sc, uint16_t* out)
{
    constexpr int NR = D == 3 ? 3 : 2;
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < E;
         e += gridDim.x * blockDim.x) {
        const uint32_t i = recv[e], j = send[e];
        float4 a[NR], b[NR];
        for (int q = 0; q < NR; q++) {
            a[q] = rec[(size_t)i * NR + q];
            b[q] = rec[(size_t)j * NR + q];
        }
        float ri[3], rj[3], ui[3], uj[3], nj[3];
        float rhoi, rhoj;
        int imj;
        if (D == 2) {
            ri[0] = a[0].x; ri[1] = a[0].y; ui[0] = a[0].z; ui[1] = a[0].w;
            rj[0] = b[0].x; rj[1] = b[0].y; uj[0] = b[0].z; uj[1] = b[0].w;
            rhoi = a[1].x;
            rhoj = b[1].x;
            imj = __float_as_int(b[1].y);
            nj[0] = b[1].z; nj[1] = b[1].w;
        } else {
            ri[0] = a[0].x; ri[1] = a[0].y; ri[2] = a[0].z; rhoi = a[0].w;
            rj[0] = b[0].x; rj[1] = b[0].y; rj[2] = b[0].z; rhoj = b[0].w;
            ui[0] = a[1].x; ui[1] = a[1].y; ui[2] = a[1].z;
            uj[0] = b[1].x; uj[1] = b[1].y; uj[2] = b[1].z;
            imj = __float_as_int(b[1].w);
            nj[0] = b[2].x; nj[1] = b[2].y; nj[2] = b[2].z;
        }
        float f[AQUA_GNN_FEATURES];
        for (int k = 0; k < AQUA_GNN_FEATURES; k++)
            f[k] = 0.f;
        const float h = sc[0], U = sc[1], R = sc[2];
        int k = 0;
        float rr = 0.f;
        for (int d = 0; d < D; d++) {
            const float dd = rj[d] - ri[d];
            rr += dd * dd;
            f[k++] = dd / h;
        }
        const float q = sqrtf(rr) / h;
        f[k++] = q;
        for (int d = 0; d < D; d++)
            f[k++] = (uj[d] - ui[d]) / U;
        f[k++] = (rhoj - rhoi) / R;
        f[k++] = wendland_shape(q);
        const bool wall = imj < 0;
        f[k++] = wall ? 1.f : 0.f;
        for (int d = 0; d < D; d++)
            f[k++] = wall ? nj[d] : 0.f;
        // the 32-byte row as two 16-byte stores
        uint4* row = reinterpret_cast<uint4*>(out + (size_t)e * AQUA_GNN_FEATURES);
        row[0] = make_uint4(pack_bf2(f[0], f[1]), pack_bf2(f[2], f[3]),
                            pack_bf2(f[4], f[5]), pack_bf2(f[6], f[7]));
        row[1] = make_uint4(pack_bf2(f[8], f[9]), pack_bf2(f[10], f[11]),
                            pack_bf2(f[12], f[13]), pack_bf2(f[14], f[15]));
    }
}

// ---------------------------------------------------------- dense layers ----

constexpr int kLinThreads = 128;  // 4 warps, 16 rows each per tile
constexpr int kMaxK = 160;

// Y = act(X W^T + b); W staged in shared memory as N rows of K (+8 pad)
template<int N>
__global__ void __launch_bounds__(kLinThreads)
k_linear_fwd(uint32_t M, uint32_t K, const uint16_t* __restrict__ X,
             uint32_t ldx, const uint16_t* __restrict__ W,
             const float* __restrict__ bias, float* Z, uint32_t ldz,
             uint16_t* Y, uint32_t ldy, int act)
{
    __shared__ __align__(16) uint16_t sW[N * (kMaxK + 8)];
    const uint32_t KP = K + 8;
    for (uint32_t e = threadIdx.x; e < N * K; e += kLinThreads)
        sW[(e / K) * KP + e % K] = W[e];
    __syncthreads();
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t g = lane >> 2, tq = lane & 3;
    const uint32_t tiles = (M + 15) / 16;
    for (uint32_t tile = blockIdx.x * 4 + warp; tile < tiles;
         tile += gridDim.x * 4) {
        const uint32_t r0 = tile * 16 + g, r1 = r0 + 8;
        float c[N / 8][4];
        for (int t = 0; t < N / 8; t++)
            c[t][0] = c[t][1] = c[t][2] = c[t][3] = 0.f;
        const uint16_t* x0 = X + (size_t)r0 * ldx + tq * 2;
        const uint16_t* x1 = X + (size_t)r1 * ldx + tq * 2;
        for (uint32_t k0 = 0; k0 < K; k0 += 16) {
            uint32_t a[4];
            a[0] = r0 < M ? ld_u32(x0 + k0) : 0u;
            a[1] = r1 < M ? ld_u32(x1 + k0) : 0u;
            a[2] = r0 < M ? ld_u32(x0 + k0 + 8) : 0u;
            a[3] = r1 < M ? ld_u32(x1 + k0 + 8) : 0u;
#pragma unroll
            for (int t = 0; t < N / 8; t++) {
                const uint16_t* w = sW + (t * 8 + g) * KP + k0 + tq * 2;
                const uint32_t b[2] = { ld_u32(w), ld_u32(w + 8) };
                mma_bf16(c[t], a, b);
            }
        }
#pragma unroll
        for (int t = 0; t < N / 8; t++) {
            const uint32_t col = t * 8 + tq * 2;
            const float b0 = bias ? bias[col] : 0.f;
            const float b1 = bias ? bias[col + 1] : 0.f;
            const float z[2][2] = { { c[t][0] + b0, c[t][1] + b1 },
                                    { c[t][2] + b0, c[t][3] + b1 } };
            for (int h = 0; h < 2; h++) {
                const uint32_t row = h ? r1 : r0;
                if (row >= M)
                    continue;
                if (Z)
                    *reinterpret_cast<float2*>(Z + (size_t)row * ldz + col) =
                        make_float2(z[h][0], z[h][1]);
                if (Y) {
                    const float y0 = act == AQUA_ACT_SILU ? silu(z[h][0]) : z[h][0];
                    const float y1 = act == AQUA_ACT_SILU ? silu(z[h][1]) : z[h][1];
                    *reinterpret_cast<uint32_t*>(Y + (size_t)row * ldy + col) =
                        pack_bf2(y0, y1);
                }
            }
        }
    }
}

// dX = dY W (Wt = W^T staged: K rows of N (+8)); KT = output n8 tiles
template<int KT>
__global__ void __launch_bounds__(kLinThreads)
k_linear_dgrad(uint32_t M, uint32_t N, uint32_t K,
               const uint16_t* __restrict__ dY, uint32_t ldy,
               const uint16_t* __restrict__ Wt, const float* __restrict__ Zp,
               uint32_t ldzp, int act_prev, uint16_t* dX, uint32_t ldx)
{
    __shared__ __align__(16) uint16_t sW[kMaxK * (64 + 8)];
    const uint32_t NP = N + 8;
    for (uint32_t e = threadIdx.x; e < K * N; e += kLinThreads)
        sW[(e / N) * NP + e % N] = Wt[e];
    __syncthreads();
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t g = lane >> 2, tq = lane & 3;
    const uint32_t tiles = (M + 15) / 16;
    const uint32_t kt_used = K / 8;
    for (uint32_t tile = blockIdx.x * 4 + warp; tile < tiles;
         tile += gridDim.x * 4) {
        const uint32_t r0 = tile * 16 + g, r1 = r0 + 8;
        float c[KT][4];
        for (int t = 0; t < KT; t++)
            c[t][0] = c[t][1] = c[t][2] = c[t][3] = 0.f;
        const uint16_t* y0 = dY + (size_t)r0 * ldy + tq * 2;
        const uint16_t* y1 = dY + (size_t)r1 * ldy + tq * 2;
        for (uint32_t n0 = 0; n0 < N; n0 += 16) {
            uint32_t a[4];
            a[0] = r0 < M ? ld_u32(y0 + n0) : 0u;
            a[1] = r1 < M ? ld_u32(y1 + n0) : 0u;
            a[2] = r0 < M ? ld_u32(y0 + n0 + 8) : 0u;
            a[3] = r1 < M ? ld_u32(y1 + n0 + 8) : 0u;
#pragma unroll
            for (int t = 0; t < KT; t++) {
                if ((uint32_t)t >= kt_used)
                    break;
                const uint16_t* w = sW + (t * 8 + g) * NP + n0 + tq * 2;
                const uint32_t b[2] = { ld_u32(w), ld_u32(w + 8) };
                mma_bf16(c[t], a, b);
            }
        }
#pragma unroll
        for (int t = 0; t < KT; t++) {
            if ((uint32_t)t >= kt_used)
                break;
            const uint32_t col = t * 8 + tq * 2;
            for (int h = 0; h < 2; h++) {
                const uint32_t row = h ? r1 : r0;
                if (row >= M)
                    continue;
                float v0 = c[t][2 * h], v1 = c[t][2 * h + 1];
                if (Zp && act_prev == AQUA_ACT_SILU) {
                    const float2 z = *reinterpret_cast<const float2*>(
                        Zp + (size_t)row * ldzp + col);
                    v0 *= silu_grad(z.x);
                    v1 *= silu_grad(z.y);
                }
                *reinterpret_cast<uint32_t*>(dX + (size_t)row * ldx + col) =
                    pack_bf2(v0, v1);
            }
        }
    }
}

// dW += dY^T X over row blocks of 64; warp w owns output rows [16w, 16w+16)
constexpr int kWgRows = 64;
template<int KT>
__global__ void __launch_bounds__(kLinThreads)
k_linear_wgrad(uint32_t M, uint32_t N, uint32_t K,
               const uint16_t* __restrict__ dY, uint32_t ldy,
               const uint16_t* __restrict__ X, uint32_t ldx, float* dW,
               float* db)
{
    __shared__ __align__(16) uint16_t sY[kWgRows * (64 + 8)];
    __shared__ __align__(16) uint16_t sX[kWgRows * (kMaxK + 8)];
    const uint32_t NP = 64 + 8, KP = kMaxK + 8;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t g = lane >> 2, tq = lane & 3;
    const bool active = warp * 16 < N;
    float c[KT][4];
    for (int t = 0; t < KT; t++)
        c[t][0] = c[t][1] = c[t][2] = c[t][3] = 0.f;
    float bsum = 0.f;  // column sum of dY for column threadIdx.x
    const uint32_t blocks = (M + kWgRows - 1) / kWgRows;
    const uint32_t nv = N / 8, kv = K / 8;  // 16-byte vectors per row
    for (uint32_t blk = blockIdx.x; blk < blocks; blk += gridDim.x) {
        const uint32_t m0 = blk * kWgRows;
        __syncthreads();
        for (uint32_t e = threadIdx.x; e < kWgRows * nv; e += kLinThreads) {
            const uint32_t rr = e / nv, v = e % nv;
            uint4 val = make_uint4(0, 0, 0, 0);
            if (m0 + rr < M)
                val = *reinterpret_cast<const uint4*>(dY + (size_t)(m0 + rr) * ldy + v * 8);
            *reinterpret_cast<uint4*>(sY + rr * NP + v * 8) = val;
        }
        for (uint32_t e = threadIdx.x; e < kWgRows * kv; e += kLinThreads) {
            const uint32_t rr = e / kv, v = e % kv;
            uint4 val = make_uint4(0, 0, 0, 0);
            if (m0 + rr < M)
                val = *reinterpret_cast<const uint4*>(X + (size_t)(m0 + rr) * ldx + v * 8);
            *reinterpret_cast<uint4*>(sX + rr * KP + v * 8) = val;
        }
        __syncthreads();
        if (threadIdx.x < N)
            for (int rr = 0; rr < kWgRows; rr++)
                bsum += bf2f(sY[rr * NP + threadIdx.x]);
        if (!active)
            continue;
        const uint32_t nb = warp * 16;
        const uint32_t sub = lane >> 3, i8 = lane & 7;
        for (uint32_t mb = 0; mb < (uint32_t)kWgRows; mb += 16) {
            // A = dY^T (rows n, cols m): four 8x8 blocks, transposed loads
            uint32_t a[4];
            {
                const uint32_t mrow = mb + (sub >> 1) * 8 + i8;
                const uint32_t ncol = nb + (sub & 1) * 8;
                ldsm_x4_trans(a, sY + mrow * NP + ncol);
            }
#pragma unroll
            for (int t = 0; t < KT; t += 2) {
                if ((uint32_t)t >= kv)
                    break;
                // B = X (rows m, cols k) for n8 tiles t and t+1
                uint32_t b[4];
                const uint32_t mrow = mb + (sub & 1) * 8 + i8;
                const uint32_t kcol = (t + (sub >> 1)) * 8;
                ldsm_x4_trans(b, sX + mrow * KP + (kcol < K ? kcol : 0));
                const uint32_t b0[2] = { b[0], b[1] };
                mma_bf16(c[t], a, b0);
                if ((uint32_t)t + 1 < kv) {
                    const uint32_t b1[2] = { b[2], b[3] };
                    mma_bf16(c[t + 1], a, b1);
                }
            }
        }
    }
    if (db && threadIdx.x < N)
        atomicAdd(&db[threadIdx.x], bsum);
    if (!active)
        return;
    const uint32_t nb = warp * 16;
#pragma unroll
    for (int t = 0; t < KT; t++) {
        if ((uint32_t)t >= kv)
            break;
        const uint32_t col = t * 8 + tq * 2;
        atomicAdd(&dW[(size_t)(nb + g) * K + col], c[t][0]);
        atomicAdd(&dW[(size_t)(nb + g) * K + col + 1], c[t][1]);
        atomicAdd(&dW[(size_t)(nb + g + 8) * K + col], c[t][2]);
        atomicAdd(&dW[(size_t)(nb + g + 8) * K + col + 1], c[t][3]);
    }
}

// ----------------------------------------------------------- aggregation ----

// warp per node; lane l sums columns 2l, 2l+1
__global__ void
k_segment_sum(uint32_t n, const uint32_t* __restrict__ off,
              const uint16_t* __restrict__ Y, uint32_t ldy, float scale,
              uint16_t* out, uint32_t ld, uint32_t col)
{
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < n;
         s += (gridDim.x * blockDim.x) >> 5) {
        float a0 = 0.f, a1 = 0.f;
        const uint32_t b = off[s], e = off[s + 1];
        for (uint32_t k = b; k < e; k++) {
            const uint32_t v = ld_u32(Y + (size_t)k * ldy + 2 * lane);
            a0 += bf2f((uint16_t)(v & 0xffffu));
            a1 += bf2f((uint16_t)(v >> 16));
        }
        *reinterpret_cast<uint32_t*>(out + (size_t)s * ld + col + 2 * lane) =
            pack_bf2(a0 * scale, a1 * scale);
    }
}

__global__ void
k_segment_bcast(uint32_t E, const uint32_t* __restrict__ recv,
                const uint16_t* __restrict__ dA, uint32_t ld, uint32_t col,
                float scale, uint16_t* dY, uint32_t ldy)
{
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < E;
         e += (gridDim.x * blockDim.x) >> 5) {
        const uint32_t v = ld_u32(dA + (size_t)recv[e] * ld + col + 2 * lane);
        const float a0 = bf2f((uint16_t)(v & 0xffffu)) * scale;
        const float a1 = bf2f((uint16_t)(v >> 16)) * scale;
        *reinterpret_cast<uint32_t*>(dY + (size_t)e * ldy + 2 * lane) =
            pack_bf2(a0, a1);
    }
}

// row e: [H[recv], H[send], E] -> 144 bf16 = 18 vectors of 8
__global__ void
k_gather_pair(uint32_t En, const uint32_t* __restrict__ recv,
              const uint32_t* __restrict__ send, const uint16_t* __restrict__ H,
              uint32_t ldh, const uint16_t* __restrict__ Ef, uint16_t* out)
{
    const uint64_t total = (uint64_t)En * 18;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
         t < total; t += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t e = (uint32_t)(t / 18), v = (uint32_t)(t % 18);
        uint4 val;
        if (v < 8)
            val = *reinterpret_cast<const uint4*>(H + (size_t)recv[e] * ldh + v * 8);
        else if (v < 16)
            val = *reinterpret_cast<const uint4*>(H + (size_t)send[e] * ldh + (v - 8) * 8);
        else
            val = *reinterpret_cast<const uint4*>(Ef + (size_t)e * AQUA_GNN_FEATURES + (v - 16) * 8);
        *reinterpret_cast<uint4*>(out + (size_t)e * 144 + v * 8) = val;
    }
}

// receiver half: warp per node, no atomics; sender half: atomics per edge
__global__ void
k_scatter_pair_recv(uint32_t n, const uint32_t* __restrict__ off,
                    const uint16_t* __restrict__ dX, float* dH)
{
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < n;
         s += (gridDim.x * blockDim.x) >> 5) {
        float a0 = 0.f, a1 = 0.f;
        for (uint32_t k = off[s]; k < off[s + 1]; k++) {
            const uint32_t v = ld_u32(dX + (size_t)k * 144 + 2 * lane);
            a0 += bf2f((uint16_t)(v & 0xffffu));
            a1 += bf2f((uint16_t)(v >> 16));
        }
        float2* p = reinterpret_cast<float2*>(dH + (size_t)s * 64 + 2 * lane);
        float2 o = *p;
        o.x += a0;
        o.y += a1;
        *p = o;
    }
}

__global__ void
k_scatter_pair_send(uint32_t En, const uint32_t* __restrict__ send,
                    const uint16_t* __restrict__ dX, float* dH)
{
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < En;
         e += (gridDim.x * blockDim.x) >> 5) {
        const uint32_t v = ld_u32(dX + (size_t)e * 144 + 64 + 2 * lane);
        float* p = dH + (size_t)send[e] * 64 + 2 * lane;
        atomicAdd(p, bf2f((uint16_t)(v & 0xffffu)));
        atomicAdd(p + 1, bf2f((uint16_t)(v >> 16)));
    }
}

__global__ void
k_add_to_bf16(uint32_t n, const float* __restrict__ src,
              const uint16_t* __restrict__ extra, uint32_t eld, uint32_t ecol,
              uint16_t* dst, uint32_t ld, uint32_t col)
{
    const uint64_t total = (uint64_t)n * 32;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
         t < total; t += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t s = (uint32_t)(t / 32), c = (uint32_t)(t % 32) * 2;
        float a0 = src[(size_t)s * 64 + c], a1 = src[(size_t)s * 64 + c + 1];
        if (extra) {
            const uint32_t v = ld_u32(extra + (size_t)s * eld + ecol + c);
            a0 += bf2f((uint16_t)(v & 0xffffu));
            a1 += bf2f((uint16_t)(v >> 16));
        }
        *reinterpret_cast<uint32_t*>(dst + (size_t)s * ld + col + c) = pack_bf2(a0, a1);
    }
}

// ------------------------------------------------------ loss / optimiser ----

__global__ void
k_mse(uint32_t n, uint32_t t, const float* __restrict__ out,
      const float* __restrict__ target, const int32_t* __restrict__ mask,
      float inv_count, float* loss, uint16_t* dOut)
{
    float acc = 0.f;
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n;
         s += gridDim.x * blockDim.x) {
        uint16_t* row = dOut + (size_t)s * 16;
        for (int c = 0; c < 16; c += 2)
            *reinterpret_cast<uint32_t*>(row + c) = 0u;
        if (!mask[s])
            continue;
        for (uint32_t c = 0; c < t; c++) {
            const float d = out[(size_t)s * 16 + c] - target[(size_t)s * t + c];
            acc += d * d;
            row[c] = f2bf(2.f * d * inv_count);
        }
    }
    for (int o = 16; o > 0; o >>= 1)
        acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0 && acc != 0.f)
        atomicAdd(loss, acc * inv_count);
}

__global__ void
k_adam(uint32_t n, float* w, const float* __restrict__ g, float* m, float* v,
       float lr, float b1, float b2, float eps, float c1, float c2,
       uint16_t* wb)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float mh = mi / c1, vh = vi / c2;
        const float wi = w[i] - lr * mh / (sqrtf(vh) + eps);
        w[i] = wi;
        if (wb)
            wb[i] = f2bf(wi);
    }
}

__global__ void
k_to_bf16(uint32_t n, const float* __restrict__ src, uint16_t* dst)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x)
        dst[i] = f2bf(src[i]);
}

__global__ void
k_transpose(uint32_t N, uint32_t K, const uint16_t* __restrict__ W,
            uint16_t* Wt)
{
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < N * K;
         e += gridDim.x * blockDim.x) {
        const uint32_t nn = e / K, k = e % K;
        Wt[(size_t)k * N + nn] = W[e];
    }
}

// ------------------------------------------------------------- proposal ----

__global__ void
k_apply(uint32_t n, int dims, const uint32_t* __restrict__ perm,
        const float* __restrict__ out, const uint32_t* __restrict__ cid,
        const float* __restrict__ dt_case, uint32_t k, float su, float srho,
        float* r, float* u, float* rho, const float* __restrict__ dudt,
        const float* __restrict__ drhodt, const int32_t* __restrict__ imove)
{
    const uint32_t VS = dims == 3 ? 4 : 2;
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n;
         s += gridDim.x * blockDim.x) {
        const uint32_t i = perm[s];
        if (imove[i] != 1)
            continue;
        const float T = (float)k * dt_case[cid[i]];
        for (int d = 0; d < dims; d++) {
            const size_t q = (size_t)i * VS + d;
            const float u0 = u[q];
            const float u1 = u0 + T * dudt[q] + su * out[(size_t)s * 16 + d];
            u[q] = u1;
            r[q] = r[q] + T * 0.5f * (u0 + u1);
        }
        rho[i] = rho[i] + T * drhodt[i] + srho * out[(size_t)s * 16 + dims];
    }
}

__global__ void
k_targets(uint32_t n, int dims, const uint32_t* __restrict__ perm,
          const float* __restrict__ u0, const float* __restrict__ rho0,
          const float* __restrict__ dudt0, const float* __restrict__ drhodt0,
          const float* __restrict__ u1, const float* __restrict__ rho1,
          const uint32_t* __restrict__ cid, const float* __restrict__ dt_case,
          uint32_t k, float su, float srho, const int32_t* __restrict__ imove,
          float* target, int32_t* mask)
{
    const uint32_t VS = dims == 3 ? 4 : 2;
    const uint32_t t = dims + 1;
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n;
         s += gridDim.x * blockDim.x) {
        const uint32_t i = perm[s];
        const bool fluid = imove[i] == 1;
        mask[s] = fluid ? 1 : 0;
        const float T = (float)k * dt_case[cid[i]];
        for (int d = 0; d < dims; d++) {
            const size_t q = (size_t)i * VS + d;
            target[(size_t)s * t + d] =
                fluid ? (u1[q] - u0[q] - T * dudt0[q]) / su : 0.f;
        }
        target[(size_t)s * t + dims] =
            fluid ? (rho1[i] - rho0[i] - T * drhodt0[i]) / srho : 0.f;
    }
}

__global__ void
k_roll(uint32_t n, int dims, const uint32_t* __restrict__ cid,
       const uint32_t* __restrict__ iset, const int32_t* __restrict__ imove,
       const int32_t* __restrict__ enabled, const uint32_t* __restrict__ rset,
       const float* __restrict__ psi0, const float* __restrict__ psi1,
       const float* __restrict__ omega1, const float* __restrict__ center,
       float* r, float* nrm, float* tng, float* u)
{
    const uint32_t VS = dims == 3 ? 4 : 2;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        const uint32_t c = cid[i];
        if (!enabled[c] || imove[i] == 1 || iset[i] != rset[c])
            continue;
        const double dpsi = (double)psi1[c] - (double)psi0[c];
        const float cs = (float)cos(dpsi), sn = (float)sin(dpsi);
        const float cx = center[4 * c], cy = center[4 * c + 1];
        const size_t q = (size_t)i * VS;
        const float x = r[q] - cx, y = r[q + 1] - cy;
        const float xr = cs * x - sn * y, yr = sn * x + cs * y;
        r[q] = xr + cx;
        r[q + 1] = yr + cy;
        float a = nrm[q], b = nrm[q + 1];
        nrm[q] = cs * a - sn * b;
        nrm[q + 1] = sn * a + cs * b;
        a = tng[q];
        b = tng[q + 1];
        tng[q] = cs * a - sn * b;
        tng[q + 1] = sn * a + cs * b;
        u[q] = -omega1[c] * yr;
        u[q + 1] = omega1[c] * xr;
    }
}

// warp per case: locate the first probe, then lanes sum over the case
template<int D>
__global__ void
k_probe_pressure(uint32_t n_cases, const uint32_t* __restrict__ off,
                 const float* __restrict__ r, const float* __restrict__ rho,
                 const float* __restrict__ m, const int32_t* __restrict__ imove,
                 float H, float CONW, float SUPPORT, float cs, float p0,
                 float refd, float* out)
{
    constexpr int VS = D == 3 ? 4 : 2;
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < n_cases;
         c += (gridDim.x * blockDim.x) >> 5) {
        const uint32_t lo = off[c], hi = off[c + 1];
        uint32_t probe = 0xffffffffu;
        for (uint32_t b = lo; b < hi && probe == 0xffffffffu; b += 32) {
            const bool is = b + lane < hi && imove[b + lane] == 0;
            const uint32_t bal = __ballot_sync(0xffffffffu, is);
            if (bal)
                probe = b + (__ffs(bal) - 1);
        }
        if (probe == 0xffffffffu) {
            if (lane == 0)
                out[c] = 0.f;
            continue;
        }
        float pr[3];
        for (int d = 0; d < D; d++)
            pr[d] = r[(size_t)probe * VS + d];
        float sp = 0.f, sw = 0.f;
        for (uint32_t j = lo + lane; j < hi; j += 32) {
            if (imove[j] != 1)
                continue;
            float rr = 0.f;
            for (int d = 0; d < D; d++) {
                const float dd = r[(size_t)j * VS + d] - pr[d];
                rr += dd * dd;
            }
            const float q = sqrtf(rr) / H;
            if (q >= SUPPORT)
                continue;
            const float a = 2.f - q;
            const float wq = (D == 3 ? 0.08203125f : 0.109375f) * 0.318309886f *
                             (1.f + 2.f * q) * a * a * a * a;
            const float w = wq * CONW * m[j] / rho[j];
            sw += w;
            sp += (p0 + cs * cs * (rho[j] - refd)) * w;
        }
        for (int o = 16; o > 0; o >>= 1) {
            sp += __shfl_xor_sync(0xffffffffu, sp, o);
            sw += __shfl_xor_sync(0xffffffffu, sw, o);
        }
        if (lane == 0)
            out[c] = sp / (sw < 1.0e-6f ? 1.f : sw);
    }
}

// Several probes of one large case: fixed grid, each thread sums its
// grid-stride particles for every probe, the blocks reduce in a fixed tree
// and a last kernel adds the blocks' partials in block order, so the result
// does not depend on scheduling.
constexpr int kProbeBlocks = AQUA_GNN_PROBE_BLOCKS;
constexpr int kProbeThreads = 256;

template<int D>
__global__ void __launch_bounds__(kProbeThreads)
k_probes_partial(uint32_t n, const float* __restrict__ r,
                 const float* __restrict__ rho, const float* __restrict__ m,
                 const int32_t* __restrict__ imove, uint32_t n_probes,
                 const uint32_t* __restrict__ probe, float H, float CONW,
                 float SUPPORT, float cs, float p0, float refd, float* partial)
{
    constexpr int VS = D == 3 ? 4 : 2;
    constexpr uint32_t P = AQUA_GNN_MAX_PROBES;
    __shared__ float red[2][kProbeThreads];
    float pr[P][3];
    float sp[P], sw[P];
    for (uint32_t k = 0; k < P; k++) {
        sp[k] = sw[k] = 0.f;
        for (int d = 0; d < 3; d++)
            pr[k][d] = (k < n_probes && d < D) ? r[(size_t)probe[k] * VS + d] : 0.f;
    }
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n;
         j += gridDim.x * blockDim.x) {
        if (imove[j] != 1)
            continue;
        float rj[3];
        for (int d = 0; d < D; d++)
            rj[d] = r[(size_t)j * VS + d];
        const float w0 = CONW * m[j] / rho[j];
        const float pj = p0 + cs * cs * (rho[j] - refd);
        for (uint32_t k = 0; k < P; k++) {
            if (k >= n_probes)
                break;
            float rr = 0.f;
            for (int d = 0; d < D; d++) {
                const float dd = rj[d] - pr[k][d];
                rr += dd * dd;
            }
            const float q = sqrtf(rr) / H;
            if (q >= SUPPORT)
                continue;
            const float a = 2.f - q;
            const float wq = (D == 3 ? 0.08203125f : 0.109375f) * 0.318309886f *
                             (1.f + 2.f * q) * a * a * a * a;
            const float w = wq * w0;
            sw[k] += w;
            sp[k] += pj * w;
        }
    }
    for (uint32_t k = 0; k < n_probes && k < P; k++) {
        red[0][threadIdx.x] = sp[k];
        red[1][threadIdx.x] = sw[k];
        __syncthreads();
        for (int o = kProbeThreads / 2; o > 0; o >>= 1) {
            if ((int)threadIdx.x < o) {
                red[0][threadIdx.x] += red[0][threadIdx.x + o];
                red[1][threadIdx.x] += red[1][threadIdx.x + o];
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            partial[(size_t)(2 * k) * kProbeBlocks + blockIdx.x] = red[0][0];
            partial[(size_t)(2 * k + 1) * kProbeBlocks + blockIdx.x] = red[1][0];
        }
        __syncthreads();
    }
}

__global__ void
k_probes_final(uint32_t n_probes, const float* __restrict__ partial, float* out)
{
    const uint32_t k = threadIdx.x;
    if (k >= n_probes)
        return;
    float sp = 0.f, sw = 0.f;
    for (int b = 0; b < kProbeBlocks; b++) {
        sp += partial[(size_t)(2 * k) * kProbeBlocks + b];
        sw += partial[(size_t)(2 * k + 1) * kProbeBlocks + b];
    }
    out[k] = sp / (sw < 1.0e-6f ? 1.f : sw);
}

// 32-bit integer hash (the "lowbias32" mixer: xor-shift / multiply rounds)
__device__ __forceinline__ uint32_t
mix32(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

// max |a_i - b_i| * scale over the fluid particles whose hash of (i, seed)
// falls below `below` (a Bernoulli subsample of fraction below / 2^32); a
// non-finite difference counts as infinite.  The maximum of non-negative
// floats is taken on their bit patterns with atomicMax: order-independent.
__global__ void
k_sample_max_diff(uint32_t n, const float* __restrict__ a,
                  const float* __restrict__ b, const int32_t* __restrict__ imove,
                  uint32_t seed, uint32_t below, float scale, int* out)
{
    float mx = 0.f;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        if (imove[i] != 1 || mix32(i ^ mix32(seed)) >= below)
            continue;
        float d = fabsf(a[i] - b[i]) * scale;
        if (!(d <= 3.0e38f))
            d = INFINITY;
        mx = fmaxf(mx, d);
    }
    for (int o = 16; o > 0; o >>= 1)
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0 && mx > 0.f)
        atomicMax(out, __float_as_int(mx));
}

// The rate-sample judge of a proposal (see aqua_gnn_judge_density)
__global__ void
k_judge_density(uint32_t n, const uint32_t* __restrict__ id1,
                const uint32_t* __restrict__ icell1,
                const int32_t* __restrict__ imove1,
                const float* __restrict__ drhodt1,
                const uint32_t* __restrict__ icell0,
                const float* __restrict__ drhodt0,
                const float* __restrict__ rho0, const float* __restrict__ rho1,
                float half_kdt, float scale, uint32_t below, uint32_t seed,
                float* __restrict__ rho_judged, int* out)
{
    float mx = 0.f;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        const uint32_t o = id1[i];
        const bool both = aqua::sample_hash(icell1[i], seed) < below &&
                          aqua::sample_hash(icell0[o], seed) < below;
        const float rj = rho0[o] + half_kdt * (drhodt0[o] + drhodt1[i]);
        rho_judged[o] = rj;
        if (imove1[i] != 1 || !both)
            continue;
        float d = fabsf(rho1[o] - rj) * scale;
        if (!(d <= 3.0e38f))
            d = INFINITY;
        mx = fmaxf(mx, d);
    }
    for (int o = 16; o > 0; o >>= 1)
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0 && mx > 0.f)
        atomicMax(out, __float_as_int(mx));
}

__global__ void
k_case_max_diff(uint32_t n_cases, const uint32_t* __restrict__ off,
                const float* __restrict__ a, const float* __restrict__ b,
                const int32_t* __restrict__ imove, float scale, float* out)
{
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < n_cases;
         c += (gridDim.x * blockDim.x) >> 5) {
        float mx = 0.f;
        for (uint32_t j = off[c] + lane; j < off[c + 1]; j += 32)
            if (imove[j] == 1)
                mx = fmaxf(mx, fabsf(a[j] - b[j]) * scale);
        for (int o = 16; o > 0; o >>= 1)
            mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (lane == 0)
            out[c] = mx;
    }
}

}  // namespace

// ================================================================ C ABI ====

extern "C" {

aqua_status
aqua_gnn_cell_keys(uint32_t n, int32_t dims, const float* r,
                   const int32_t* imove, const uint32_t* cid, float cell,
                   const float* o, const uint32_t* nc, uint32_t* keys,
                   uint32_t* vals, void* stream)
{
    if ((dims != 2 && dims != 3) || !r || !imove || !cid || !o || !nc ||
        !keys || !vals || !(cell > 0.f))
        return AQUA_ERR_INVALID;
    const uint64_t per_case = (uint64_t)nc[0] * nc[1] * (dims == 3 ? nc[2] : 1u);
    if (per_case == 0 || per_case > 0xffffffffull)
        return AQUA_ERR_INVALID;
    if (n == 0)
        return AQUA_OK;
    k_cell_keys<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
        n, dims, r, imove, cid, cell, o[0], o[1], dims == 3 ? o[2] : 0.f, nc[0],
        nc[1], dims == 3 ? nc[2] : 1u, keys, vals);
    return last_error();
}

aqua_status
aqua_gnn_cell_ranges(uint32_t n, const uint32_t* k, uint32_t n_keys,
                     uint32_t* start, uint32_t* end, void* stream)
{
    if (!k || !start || !end)
        return AQUA_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    k_fill_u32<<<blocks_for(n_keys, 256), 256, 0, s>>>(n_keys, 0u, start);
    k_fill_u32<<<blocks_for(n_keys, 256), 256, 0, s>>>(n_keys, 0u, end);
    if (n)
        k_cell_ranges<<<blocks_for(n, 256), 256, 0, s>>>(n, k, n_keys, start, end);
    return last_error();
}

aqua_status
aqua_gnn_neighbours(uint32_t n, int32_t dims, const float* rs,
                    const uint32_t* keys, const uint32_t* nc,
                    const uint32_t* cstart, const uint32_t* cend, float radius,
                    uint32_t* degree, const uint32_t* offsets,
                    uint32_t* receivers, uint32_t* senders, void* stream)
{
    if ((dims != 2 && dims != 3) || !rs || !keys || !nc || !cstart || !cend ||
        !(radius > 0.f))
        return AQUA_ERR_INVALID;
    if (senders ? (!offsets || !receivers) : !degree)
        return AQUA_ERR_INVALID;
    if (n == 0)
        return AQUA_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const float r2 = radius * radius;
    if (dims == 3)
        k_neighbours<3><<<blocks_for(n, 128), 128, 0, s>>>(
            n, rs, keys, nc[0], nc[1], nc[2], cstart, cend, r2, degree, offsets,
            receivers, senders);
    else
        k_neighbours<2><<<blocks_for(n, 128), 128, 0, s>>>(
            n, rs, keys, nc[0], nc[1], 1u, cstart, cend, r2, degree, offsets,
            receivers, senders);
    return last_error();
}

aqua_status
aqua_gnn_bbox(uint32_t n, int32_t dims, const float* r, const int32_t* imove,
              int32_t* scratch, float* out, void* stream)
{
    if ((dims != 2 && dims != 3) || !r || !imove || !scratch || !out)
        return AQUA_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    k_bbox_init<<<1, 32, 0, s>>>(scratch);
    if (n)
        k_bbox<<<blocks_for(n, 256, 152u * 8u), 256, 0, s>>>(n, dims, r, imove,
                                                             scratch);
    float* dev = reinterpret_cast<float*>(scratch);   // decoded in place
    k_bbox_decode<<<1, 32, 0, s>>>(scratch, dev);
    if (cudaMemcpyAsync(out, dev, 6 * sizeof(float), cudaMemcpyDeviceToHost, s) !=
            cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return AQUA_ERR_CUDA;
    return last_error();
}

aqua_status
aqua_gnn_exclusive_scan(uint32_t n, const uint32_t* in, uint32_t* out,
                        uint32_t* scratch, void* stream)
{
    if (!in || !out || !scratch || n > (1u << 26))
        return AQUA_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles > (uint32_t)kScanThreads * 16)
        return AQUA_ERR_INVALID;
    uint32_t* sums = scratch;
    uint32_t* grand = scratch + (tiles > 0 ? tiles : 1);
    if (n > 0)
        k_scan_tiles<<<tiles, kScanThreads, 0, s>>>(n, in, out, sums);
    k_scan_sums<<<1, kScanThreads, 0, s>>>(tiles, sums, grand);
    k_scan_add<<<blocks_for((uint64_t)n + 1, 256), 256, 0, s>>>(n, out, sums, grand);
    return last_error();
}

aqua_status
aqua_gnn_gather32(uint32_t n, const uint32_t* perm, const void* src,
                  uint32_t stride, uint32_t comps, void* dst, void* stream)
{
    if (!perm || !src || !dst || comps == 0 || stride < comps)
        return AQUA_ERR_INVALID;
    if (n == 0)
        return AQUA_OK;
    k_gather32<<<blocks_for((uint64_t)n * comps, 256), 256, 0,
                 (cudaStream_t)stream>>>(n, perm, (const uint32_t*)src, stride,
                                         comps, (uint32_t*)dst);
    return last_error();
}

aqua_status
aqua_gnn_scatter32(uint32_t n, const uint32_t* perm, const void* src,
                   uint32_t comps, void* dst, uint32_t stride, void* stream)
{
    if (!perm || !src || !dst || comps == 0 || stride < comps)
        return AQUA_ERR_INVALID;
    if (n == 0)
        return AQUA_OK;
    k_scatter32<<<blocks_for((uint64_t)n * comps, 256), 256, 0,
                  (cudaStream_t)stream>>>(n, perm, (const uint32_t*)src, comps,
                                          (uint32_t*)dst, stride);
    return last_error();
}

aqua_status
aqua_gnn_node_features(uint32_t n, int32_t dims, const float* u,
                       const float* rho, const float* dudt, const float* drhodt,
                       const int32_t* imove, const float* normal,
                       const float* scales, uint16_t* out, uint32_t ld,
                       uint32_t col, void* stream)
{
    if ((dims != 2 && dims != 3) || !u || !rho || !dudt || !drhodt || !imove ||
        !normal || !scales || !out || ld % 8 || col % 8 ||
        col + AQUA_GNN_FEATURES > ld)
        return AQUA_ERR_INVALID;
    if (n == 0)
        return AQUA_OK;
    k_node_features<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
        n, dims, u, rho, dudt, drhodt, imove, normal, scales, out, ld, col);
    return last_error();
}

aqua_status
aqua_gnn_edge_features(uint32_t E, int32_t dims, const uint32_t* recv,
                       const uint32_t* send, const float* r, const float* u,
                       const float* rho, const int32_t* imove,
                       const float* normal, const float* scales, uint16_t* out,
                       void* stream)
{
    if ((dims != 2 && dims != 3) || !recv || !send || !r || !u || !rho ||
        !imove || !normal || !scales || !out)
        return AQUA_ERR_INVALID;
    if (E == 0)
        return AQUA_OK;
    k_edge_features<<<blocks_for(E, 256), 256, 0, (cudaStream_t)stream>>>(
        E, dims, recv, send, r, u, rho, imove, normal, scales, out);
    return last_error();
}

aqua_status
aqua_gnn_node_records(uint32_t n, int32_t dims, const float* r, const float* u,
                      const float* rho, const int32_t* imove,
                      const float* normal, float* rec, void* stream)
{
    if ((dims != 2 && dims != 3) || !r || !u || !rho || !imove || !normal ||
        !rec || (reinterpret_cast<uintptr_t>(rec) & 15))
        return AQUA_ERR_INVALID;
    if (n == 0)
        return AQUA_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (dims == 3)
        k_node_records<3><<<blocks_for(n, 256), 256, 0, s>>>(
            n, r, u, rho, imove, normal, reinterpret_cast<float4*>(rec));
    else
        k_node_records<2><<<blocks_for(n, 256), 256, 0, s>>>(
            n, r, u, rho, imove, normal, reinterpret_cast<float4*>(rec));
    return last_error();
}

aqua_status
aqua_gnn_edge_features_rec(uint32_t E, int32_t dims, const uint32_t* recv,
                           const uint32_t* send, const float* rec,
                           const float* scales, uint16_t* out, void* stream)
{
    if ((dims != 2 && dims != 3) || !recv || !send || !rec || !scales ||
        !out || (reinterpret_cast<uintptr_t>(rec) & 15) ||
        (reinterpret_cast<uintptr_t>(out) & 15))
        return AQUA_ERR_INVALID;
    if (E == 0)
        return AQUA_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const float4* r4 = reinterpret_cast<const float4*>(rec);
    if (dims == 3)
        k_edge_features_rec<3><<<blocks_for(E, 256), 256, 0, s>>>(
            E, recv, send, r4, scales, out);
    else
        k_edge_features_rec<2><<<blocks_for(E, 256), 256, 0, s>>>(
            E, recv, send, r4, scales, out);
    return last_error();
}

aqua_status
aqua_gnn_linear_fwd(uint32_t M, uint32_t K, uint32_t N, const uint16_t* X,
                    uint32_t ldx, const uint16_t* W, const float* b, float* Z,
                    uint32_t ldz, uint16_t* Y, uint32_t ldy, int32_t act,
                    void* stream)
{
    if (!X || !W || (!Z && !Y) || K == 0 || K % 16 || K > (uint32_t)kMaxK ||
        (N != 16 && N != 64) || ldx < K || ldx % 8 || (Z && (ldz < N || ldz % 2)) ||
        (Y && (ldy < N || ldy % 8)))
        return AQUA_ERR_INVALID;
    if (M == 0)
        return AQUA_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const unsigned grid = blocks_for((M + 15) / 16, 4, 152u * 16u);
    if (N == 64)
        k_linear_fwd<64><<<grid, kLinThreads, 0, s>>>(M, K, X, ldx, W, b, Z,
                                                       ldz, Y, ldy, act);
    else
        k_linear_fwd<16><<<grid, kLinThreads, 0, s>>>(M, K, X, ldx, W, b, Z,
                                                       ldz, Y, ldy, act);
    return last_error();
}

aqua_status
aqua_gnn_linear_dgrad(uint32_t M, uint32_t N, uint32_t K, const uint16_t* dY,
                      uint32_t ldy, const uint16_t* Wt, const float* Zp,
                      uint32_t ldzp, int32_t act_prev, uint16_t* dX,
                      uint32_t ldx, void* stream)
{
    if (!dY || !Wt || !dX || N == 0 || N % 16 || N > 64 || K == 0 || K % 16 ||
        K > (uint32_t)kMaxK || ldy < N || ldy % 8 || ldx < K || ldx % 8 ||
        (Zp && (ldzp < K || ldzp % 2)))
        return AQUA_ERR_INVALID;
    if (M == 0)
        return AQUA_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const unsigned grid = blocks_for((M + 15) / 16, 4, 152u * 16u);
    k_linear_dgrad<kMaxK / 8><<<grid, kLinThreads, 0, s>>>(
        M, N, K, dY, ldy, Wt, Zp, ldzp, act_prev, dX, ldx);
    return last_error();
}

aqua_status
aqua_gnn_linear_wgrad(uint32_t M, uint32_t N, uint32_t K, const uint16_t* dY,
                      uint32_t ldy, const uint16_t* X, uint32_t ldx, float* dW,
                      float* db, void* stream)
{
    if (!dY || !X || !dW || (N != 16 && N != 64) || K == 0 || K % 16 ||
        K > (uint32_t)kMaxK || ldy < N || ldy % 8 || ldx < K || ldx % 8)
        return AQUA_ERR_INVALID;
    if (M == 0)
        return AQUA_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const unsigned grid = blocks_for((M + kWgRows - 1) / kWgRows, 1, 152u * 4u);
    k_linear_wgrad<kMaxK / 8><<<grid, kLinThreads, 0, s>>>(M, N, K, dY, ldy, X,
                                                           ldx, dW, db);
    return last_error();
}

aqua_status
aqua_gnn_segment_sum(uint32_t n, const uint32_t* off, const uint16_t* Y,
                     uint32_t ldy, float scale, uint16_t* out, uint32_t ld,
                     uint32_t col, void* stream)
{
    if (!off || !Y || !out || ldy < 64 || ldy % 8 || ld % 8 || col % 8 ||
        col + 64 > ld)
        return AQUA_ERR_INVALID;
    if (n == 0)
        return AQUA_OK;
    k_segment_sum<<<blocks_for((uint64_t)n * 32, 256), 256, 0,
                    (cudaStream_t)stream>>>(n, off, Y, ldy, scale, out, ld, col);
    return last_error();
}

aqua_status
aqua_gnn_segment_bcast(uint32_t E, const uint32_t* recv, const uint16_t* dA,
                       uint32_t ld, uint32_t col, float scale, uint16_t* dY,
                       uint32_t ldy, void* stream)
{
    if (!recv || !dA || !dY || ld % 8 || col % 8 || col + 64 > ld ||
        ldy < 64 || ldy % 8)
        return AQUA_ERR_INVALID;
    if (E == 0)
        return AQUA_OK;
    k_segment_bcast<<<blocks_for((uint64_t)E * 32, 256), 256, 0,
                      (cudaStream_t)stream>>>(E, recv, dA, ld, col, scale, dY, ldy);
    return last_error();
}

aqua_status
aqua_gnn_gather_pair(uint32_t E, const uint32_t* recv, const uint32_t* send,
                     const uint16_t* H, uint32_t ldh, const uint16_t* Ef,
                     uint16_t* out, void* stream)
{
    if (!recv || !send || !H || !Ef || !out || ldh < 64 || ldh % 8)
        return AQUA_ERR_INVALID;
    if (E == 0)
        return AQUA_OK;
    k_gather_pair<<<blocks_for((uint64_t)E * 18, 256), 256, 0,
                    (cudaStream_t)stream>>>(E, recv, send, H, ldh, Ef, out);
    return last_error();
}

aqua_status
aqua_gnn_scatter_pair(uint32_t n, uint32_t E, const uint32_t* off,
                      const uint32_t* send, const uint16_t* dX, float* dH,
                      void* stream)
{
    if (!off || !send || !dX || !dH)
        return AQUA_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    if (n)
        k_scatter_pair_recv<<<blocks_for((uint64_t)n * 32, 256), 256, 0, s>>>(
            n, off, dX, dH);
    if (E)
        k_scatter_pair_send<<<blocks_for((uint64_t)E * 32, 256), 256, 0, s>>>(
            E, send, dX, dH);
    return last_error();
}

aqua_status
aqua_gnn_add_to_bf16(uint32_t n, const float* src, const uint16_t* extra,
                     uint32_t eld, uint32_t ecol, uint16_t* dst, uint32_t ld,
                     uint32_t col, void* stream)
{
    if (!src || !dst || ld % 2 || col % 2 || col + 64 > ld ||
        (extra && (eld % 2 || ecol % 2 || ecol + 64 > eld)))
        return AQUA_ERR_INVALID;
    if (n == 0)
        return AQUA_OK;
    k_add_to_bf16<<<blocks_for((uint64_t)n * 32, 256), 256, 0,
                    (cudaStream_t)stream>>>(n, src, extra, eld, ecol, dst, ld, col);
    return last_error();
}

aqua_status
aqua_gnn_mse(uint32_t n, uint32_t t, const float* out, const float* target,
             const int32_t* mask, float count, float* loss, uint16_t* dOut,
             void* stream)
{
    if (!out || !target || !mask || !loss || !dOut || t == 0 || t > 16 ||
        !(count > 0.f))
        return AQUA_ERR_INVALID;
    if (n == 0)
        return AQUA_OK;
    k_mse<<<blocks_for(n, 256, 152u * 8u), 256, 0, (cudaStream_t)stream>>>(
        n, t, out, target, mask, 1.f / count, loss, dOut);
    return last_error();
}

aqua_status
aqua_gnn_adam(uint32_t n, float* w, const float* g, float* m, float* v,
              float lr, float beta1, float beta2, float eps, uint32_t step,
              uint16_t* wb, void* stream)
{
    if (!w || !g || !m || !v || step == 0)
        return AQUA_ERR_INVALID;
    if (n == 0)
        return AQUA_OK;
    const float c1 = 1.f - powf(beta1, (float)step);
    const float c2 = 1.f - powf(beta2, (float)step);
    k_adam<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
        n, w, g, m, v, lr, beta1, beta2, eps, c1, c2, wb);
    return last_error();
}

aqua_status
aqua_gnn_to_bf16(uint32_t n, const float* src, uint16_t* dst, void* stream)
{
    if (!src || !dst)
        return AQUA_ERR_INVALID;
    if (n == 0)
        return AQUA_OK;
    k_to_bf16<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(n, src, dst);
    return last_error();
}

aqua_status
aqua_gnn_transpose(uint32_t N, uint32_t K, const uint16_t* W, uint16_t* Wt,
                   void* stream)
{
    if (!W || !Wt)
        return AQUA_ERR_INVALID;
    if (N == 0 || K == 0)
        return AQUA_OK;
    k_transpose<<<blocks_for((uint64_t)N * K, 256), 256, 0,
                  (cudaStream_t)stream>>>(N, K, W, Wt);
    return last_error();
}

aqua_status
aqua_gnn_apply(uint32_t n, int32_t dims, const uint32_t* perm, const float* out,
               const uint32_t* cid, const float* dt_case, uint32_t k, float su,
               float srho, float* r, float* u, float* rho, const float* dudt,
               const float* drhodt, const int32_t* imove, void* stream)
{
    if ((dims != 2 && dims != 3) || !perm || !out || !cid || !dt_case || !r ||
        !u || !rho || !dudt || !drhodt || !imove)
        return AQUA_ERR_INVALID;
    if (n == 0)
        return AQUA_OK;
    k_apply<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
        n, dims, perm, out, cid, dt_case, k, su, srho, r, u, rho, dudt, drhodt,
        imove);
    return last_error();
}

aqua_status
aqua_gnn_targets(uint32_t n, int32_t dims, const uint32_t* perm, const float* u0,
                 const float* rho0, const float* dudt0, const float* drhodt0,
                 const float* u1, const float* rho1, const uint32_t* cid,
                 const float* dt_case, uint32_t k, float su, float srho,
                 const int32_t* imove, float* target, int32_t* mask,
                 void* stream)
{
    if ((dims != 2 && dims != 3) || !perm || !u0 || !rho0 || !dudt0 ||
        !drhodt0 || !u1 || !rho1 || !cid || !dt_case || !imove || !target ||
        !mask || !(su > 0.f) || !(srho > 0.f))
        return AQUA_ERR_INVALID;
    if (n == 0)
        return AQUA_OK;
    k_targets<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
        n, dims, perm, u0, rho0, dudt0, drhodt0, u1, rho1, cid, dt_case, k, su,
        srho, imove, target, mask);
    return last_error();
}

aqua_status
aqua_gnn_roll(uint32_t n, int32_t dims, const uint32_t* cid,
              const uint32_t* iset, const int32_t* imove,
              const int32_t* enabled, const uint32_t* rset, const float* psi0,
              const float* psi1, const float* omega1, const float* center,
              float* r, float* normal, float* tangent, float* u, void* stream)
{
    if ((dims != 2 && dims != 3) || !cid || !iset || !imove || !enabled ||
        !rset || !psi0 || !psi1 || !omega1 || !center || !r || !normal ||
        !tangent || !u)
        return AQUA_ERR_INVALID;
    if (n == 0)
        return AQUA_OK;
    k_roll<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
        n, dims, cid, iset, imove, enabled, rset, psi0, psi1, omega1, center, r,
        normal, tangent, u);
    return last_error();
}

aqua_status
aqua_gnn_probe_pressure(uint32_t n_cases, int32_t dims, const uint32_t* off,
                        const float* r, const float* rho, const float* m,
                        const int32_t* imove, const float* k, float* out,
                        void* stream)
{
    if ((dims != 2 && dims != 3) || !off || !r || !rho || !m || !imove || !k ||
        !out)
        return AQUA_ERR_INVALID;
    if (n_cases == 0)
        return AQUA_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const unsigned g = blocks_for((uint64_t)n_cases * 32, 128);
    if (dims == 3)
        k_probe_pressure<3><<<g, 128, 0, s>>>(n_cases, off, r, rho, m, imove,
                                              k[0], k[1], k[2], k[3], k[4],
                                              k[5], out);
    else
        k_probe_pressure<2><<<g, 128, 0, s>>>(n_cases, off, r, rho, m, imove,
                                              k[0], k[1], k[2], k[3], k[4],
                                              k[5], out);
    return last_error();
}

aqua_status
aqua_gnn_case_max_diff(uint32_t n_cases, const uint32_t* off, const float* a,
                       const float* b, const int32_t* imove, float scale,
                       float* out, void* stream)
{
    if (!off || !a || !b || !imove || !out)
        return AQUA_ERR_INVALID;
    if (n_cases == 0)
        return AQUA_OK;
    k_case_max_diff<<<blocks_for((uint64_t)n_cases * 32, 128), 128, 0,
                      (cudaStream_t)stream>>>(n_cases, off, a, b, imove, scale,
                                              out);
    return last_error();
}

aqua_status
aqua_gnn_probes_pressure(uint32_t n, int32_t dims, const float* r,
                         const float* rho, const float* m,
                         const int32_t* imove, uint32_t n_probes,
                         const uint32_t* probe, const float* k, float* scratch,
                         float* out, void* stream)
{
    if ((dims != 2 && dims != 3) || !r || !rho || !m || !imove || !probe ||
        !k || !scratch || !out || n_probes > AQUA_GNN_MAX_PROBES)
        return AQUA_ERR_INVALID;
    if (n_probes == 0)
        return AQUA_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (dims == 3)
        k_probes_partial<3><<<kProbeBlocks, kProbeThreads, 0, s>>>(
            n, r, rho, m, imove, n_probes, probe, k[0], k[1], k[2], k[3], k[4],
            k[5], scratch);
    else
        k_probes_partial<2><<<kProbeBlocks, kProbeThreads, 0, s>>>(
            n, r, rho, m, imove, n_probes, probe, k[0], k[1], k[2], k[3], k[4],
            k[5], scratch);
    k_probes_final<<<1, 32, 0, s>>>(n_probes, scratch, out);
    return last_error();
}

aqua_status
aqua_gnn_sample_max_diff(uint32_t n, const float* a, const float* b,
                         const int32_t* imove, uint32_t seed, float fraction,
                         float scale, float* out, void* stream)
{
    if (!a || !b || !imove || !out || !(fraction >= 0.f && fraction <= 1.f))
        return AQUA_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    if (cudaMemsetAsync(out, 0, sizeof(float), s) != cudaSuccess)
        return AQUA_ERR_CUDA;
    if (n == 0)
        return AQUA_OK;
    const double f = (double)fraction * 4294967296.0;
    const uint32_t below = f >= 4294967295.0 ? 0xffffffffu : (uint32_t)f;
    k_sample_max_diff<<<blocks_for(n, 256, 152u * 8u), 256, 0, s>>>(
        n, a, b, imove, seed, below, scale, reinterpret_cast<int*>(out));
    return last_error();
}

aqua_status
aqua_gnn_judge_density(uint32_t n, const uint32_t* id1, const uint32_t* icell1,
                       const int32_t* imove1, const float* drhodt1,
                       const uint32_t* icell0, const float* drhodt0,
                       const float* rho0, const float* rho1, float kdt,
                       float scale, float fraction, uint32_t seed,
                       float* rho_judged, float* out, void* stream)
{
    if (!id1 || !icell1 || !imove1 || !drhodt1 || !icell0 || !drhodt0 ||
        !rho0 || !rho1 || !rho_judged || !out ||
        !(fraction > 0.f && fraction < 1.f))
        return AQUA_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    if (cudaMemsetAsync(out, 0, sizeof(float), s) != cudaSuccess)
        return AQUA_ERR_CUDA;
    if (n == 0)
        return AQUA_OK;
    // the threshold of aqua_set_rate_sample
    const uint32_t below = (uint32_t)((double)fraction * 4294967296.0);
    k_judge_density<<<blocks_for(n, 256, 152u * 8u), 256, 0, s>>>(
        n, id1, icell1, imove1, drhodt1, icell0, drhodt0, rho0, rho1,
        0.5f * kdt, scale, below, seed, rho_judged, reinterpret_cast<int*>(out));
    return last_error();
}

}  // extern "C"
