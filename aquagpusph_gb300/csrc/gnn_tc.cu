// Dense-layer forward of the learned proposal on the 5th-generation tensor
// cores: Y = act(X W^T + b) with tcgen05.mma (kind::f16, BF16 x BF16 ->
// FP32) accumulating in tensor memory.  No counterpart in the reference.
//
// One CTA of 128 threads works on tiles of 128 rows:
//   - W (N x K) is staged once in shared memory, X tiles (128 x K) per tile,
//     both in the K-major layout without swizzle: 8-row x 16-byte core
//     matrices, consecutive along K (leading byte offset 128 B), row groups
//     K/8 core matrices apart (stride byte offset);
//   - thread 0 issues K/16 MMAs of 128 x N x 16 into an N-column TMEM
//     accumulator and commits them to an mbarrier;
//   - every warp reads its 32 TMEM lanes (rows) back with tcgen05.ld, adds
//     the bias, applies the activation and stores Z (f32) and / or Y (bf16).
// Every wait on the mbarrier is bounded: on time-out the kernel records
// an error, skips the tile's stores, frees its TMEM and returns.
#include <cuda_bf16.h>
#include <atomic>
#include <cstdint>

#include "aqua_learned.h"

namespace aqua {
// test-only switch of aqua_debug_fake_timeouts() (api.cu)
extern int g_debug_fake_timeout;
}  // namespace aqua

namespace {

constexpr int kTcThreads = 128;
constexpr int kTcRows = 128;
constexpr uint32_t kWaitLimit = 1u << 22;

__device__ __forceinline__ uint32_t
smem_addr(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor: K-major, no swizzle
__device__ __forceinline__ uint64_t
make_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo & 0x3FFFFu) >> 4) << 16;
    d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version of tcgen05
    return d;                // base offset 0, swizzle none
}

// instruction descriptor of kind::f16: D f32, A and B bf16, both K-major,
// M = 128, N = n
__host__ __device__ constexpr uint32_t
make_idesc(uint32_t n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) |
           ((uint32_t)(kTcRows >> 4) << 24);
}

// SiLU of two bf16 values (a packed pair) in packed bf16 arithmetic:
// z * sigmoid(z), sigmoid(z) = (1 + tanh(z / 2)) / 2 on the hardware tanh
// (tanh.approx.bf16x2); four instructions for the pair, each result
// rounded to bf16
__device__ __forceinline__ uint32_t
silu_bf16x2(uint32_t z)
{
    const uint32_t half = 0x3f003f00u;  // 0.5 in both halves
    uint32_t h, t, s, y;
    asm("mul.rn.bf16x2 %0, %1, %2;" : "=r"(h) : "r"(z), "r"(half));
    asm("tanh.approx.bf16x2 %0, %1;" : "=r"(t) : "r"(h));
    asm("fma.rn.bf16x2 %0, %1, %2, %2;" : "=r"(s) : "r"(t), "r"(half));
    asm("mul.rn.bf16x2 %0, %1, %2;" : "=r"(y) : "r"(z), "r"(s));
    return y;
}

// two floats rounded to bf16 (round to nearest even), lo in the low half
__device__ __forceinline__ uint32_t
pack2(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

// copy a rows x K bf16 block (row-major, ld elements) into the core-matrix
// layout: element (r, k) at ((r / 8) * (K / 8) + k / 8) * 128 + (r % 8) * 16
// + (k % 8) * 2 bytes; rows past `valid` are zero
__device__ __forceinline__ void
stage(uint8_t* dst, const uint16_t* src, uint32_t ld, uint32_t rows,
      uint32_t valid, uint32_t K)
{
    const uint32_t kg = K / 8;
    for (uint32_t e = threadIdx.x; e < rows * kg; e += kTcThreads) {
        const uint32_t r = e / kg, g = e % kg;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (r < valid)
            v = *reinterpret_cast<const uint4*>(src + (size_t)r * ld + g * 8);
        *reinterpret_cast<uint4*>(dst + ((r / 8) * kg + g) * 128 + (r % 8) * 16) = v;
    }
}

template<int N>
__global__ void __launch_bounds__(kTcThreads, 1)
k_linear_fwd_tc(uint32_t M, uint32_t K, const uint16_t* __restrict__ X,
                uint32_t ldx, const uint16_t* __restrict__ W,
                const float* __restrict__ bias, float* Z, uint32_t ldz,
                uint16_t* Y, uint32_t ldy, int act, int* err, uint32_t fake)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    uint8_t* sB = smem;                                // N x K
    uint8_t* sA = smem + ((N * K * 2 + 1023) / 1024) * 1024;  // 128 x K
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    stage(sB, W, K, N, N, K);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n"
                     :: "r"(smem_addr(&mbar)));
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 "
                     "[%0], %1;\n" :: "r"(smem_addr(&tmem_base)), "r"((uint32_t)N));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    const uint32_t tmem = tmem_base;
    const uint32_t idesc = make_idesc(N);
    const uint32_t kg = K / 8;
    const uint32_t sbo = kg * 128;  // next 8-row group
    uint32_t phase = 0;
    bool failed = false;
    const uint32_t tiles = (M + kTcRows - 1) / kTcRows;
    for (uint32_t tile = blockIdx.x; tile < tiles && !failed; tile += gridDim.x) {
        const uint32_t m0 = tile * kTcRows;
        const uint32_t valid = min((uint32_t)kTcRows, M - m0);
        stage(sA, X + (size_t)m0 * ldx, ldx, kTcRows, valid, K);
        // generic-proxy stores -> visible to the tensor core (async proxy)
        asm volatile("fence.proxy.async.shared::cta;\n");
        __syncthreads();
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n");
            for (uint32_t ks = 0; ks < K / 16; ks++) {
                const uint64_t ad = make_desc(smem_addr(sA) + ks * 256, 128, sbo);
                const uint64_t bd = make_desc(smem_addr(sB) + ks * 256, 128, sbo);
                const uint32_t acc = ks > 0 ? 1u : 0u;
                asm volatile(
                    "{\n.reg .pred p;\nsetp.ne.u32 p, %4, 0;\n"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                    :: "r"(tmem), "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one."
                         "shared::cluster.b64 [%0];\n" :: "r"(smem_addr(&mbar)));
        }
        // bounded wait for the MMAs of this tile
        uint32_t done = 0;
        for (uint32_t it = 0; it < kWaitLimit && !done; it++) {
            asm volatile("{\n.reg .pred p;\n"
                         "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                         "selp.u32 %0, 1, 0, p;\n}\n"
                         : "=r"(done) : "r"(smem_addr(&mbar)), "r"(phase));
        }
        // `fake` (test switch): a wait that completed counts as timed out
        if (!__all_sync(0xffffffffu, done) || fake) {
            failed = true;
            if (lane == 0)
                atomicExch(err, 1);
        }
        failed = __syncthreads_or(failed);
        if (failed)
            break;
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;\n");
        // epilogue: warp w owns rows 32w .. 32w + 31 (TMEM lanes)
        const uint32_t row = m0 + warp * 32 + lane;
        const uint32_t taddr = tmem + ((warp * 32u) << 16);
#pragma unroll
        for (int c0 = 0; c0 < N; c0 += 16) {
            uint32_t v[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]),
                  "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]),
                  "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                  "=r"(v[14]), "=r"(v[15])
                : "r"(taddr + (uint32_t)c0));
            asm volatile("tcgen05.wait::ld.sync.aligned;\n");
            if (row < M) {
                float z[16];
                for (int j = 0; j < 16; j++)
                    z[j] = __uint_as_float(v[j]) + (bias ? bias[c0 + j] : 0.f);
                if (Z)
                    for (int j = 0; j < 16; j += 4)
                        *reinterpret_cast<float4*>(Z + (size_t)row * ldz + c0 + j) =
                            make_float4(z[j], z[j + 1], z[j + 2], z[j + 3]);
                if (Y) {
                    uint32_t p[8];
                    for (int j = 0; j < 8; j++) {
                        p[j] = pack2(z[2 * j], z[2 * j + 1]);
                        if (act == AQUA_ACT_SILU)
                            p[j] = silu_bf16x2(p[j]);
                    }
                    uint4* dst = reinterpret_cast<uint4*>(Y + (size_t)row * ldy + c0);
                    dst[0] = make_uint4(p[0], p[1], p[2], p[3]);
                    dst[1] = make_uint4(p[4], p[5], p[6], p[7]);
                }
            }
        }
        // the next tile's MMAs overwrite the accumulator and sA
        asm volatile("tcgen05.fence::before_thread_sync;\n");
        __syncthreads();
    }
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n"
                     :: "r"(tmem), "r"((uint32_t)N));
    }
}

// ---------------------------------------------------------------------------
// Fused three-layer edge MLP: Y = L3(act(L2(act(L1(X))))) on tiles of 128
// edges, every activation kept on chip.  The layer-1 input of each tile is
// gathered into shared memory (core-matrix layout) by asynchronous copies:
// rows of X, or, in PAIR mode, the concatenation [H[recv[e]] (64),
// H[send[e]] (64), Ef[e] (16)] that aqua_gnn_gather_pair materialises.  The
// three layers share one 64-column tensor-memory accumulator; each epilogue
// reads it back (tcgen05.ld), adds the bias, applies the activation, rounds
// to BF16 and writes the next layer's A operand into shared memory, exactly
// the values the unfused layers store to and reload from global memory, so
// the result is bit-identical to three aqua_gnn_linear_fwd_tc calls.  Only
// the BF16 output of layer 3 is written.  A wait that times out sets *err;
// the CTA finishes that tile (its outputs are then not to be trusted) and
// stops.
//
// With SUM the layer-3 output never leaves the chip either: it is summed
// into the receivers (aqua_gnn_segment_sum fused in).  Each CTA owns a
// contiguous range of receivers (about E / grid edges) and walks its edges
// in 128-edge tiles, in order.  The layer-3 tile is staged in shared memory
// (row-major, 16-byte groups XOR-swizzled by row), the receivers' runs of
// rows are summed by the warps (run k by warp k mod 4, lanes over column
// pairs), and a receiver whose edges continue in the next tile carries its
// partial sums there.  Every receiver's sum is thus the same sequence of
// FP32 additions, in edge order from zero, as aqua_gnn_segment_sum's: the
// output is bit-identical to the unfused kernels'.

__device__ __forceinline__ void
cp_async_16z(void* dst, const void* src, bool valid)
{
    // src-size 0 fills the 16 bytes with zeros
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n"
                 :: "r"(smem_addr(dst)), "l"(src), "r"(valid ? 16u : 0u)
                 : "memory");
}

// bytes of the operand buffer: the layer-1 input or a 128 x 64 bf16 tile
template<int K1>
__host__ __device__ constexpr uint32_t
edge_operand_bytes()
{
    constexpr uint32_t a0 = ((128u * K1 * 2u + 1023u) / 1024u) * 1024u;
    constexpr uint32_t a1 = 128u * 64u * 2u;
    return a0 > a1 ? a0 : a1;
}

// 8 warps: warps w and w + 4 read the same 32 tensor-memory lanes (rows
// 32 (w % 4) ..), each one half of the 64 columns
constexpr int kEdgeThreads = 256;
constexpr int kEdgeWarps = kEdgeThreads / 32;

// shared memory after the two operand buffers: the biases, and the
// receiver-sum bookkeeping of a SUM CTA
struct EdgeShared {
    float bias[3][64];
    uint32_t recv[kTcRows];   // receiver of each row of the tile (~0: none)
    uint32_t start[4];        // rows that start a receiver's run, per 32 rows
    float carry[2][64];       // partial sums carried into the next tile
    uint32_t carry_node[2];   // their receiver (~0: none)
    uint32_t nodes[2];        // this CTA's receivers [nodes[0], nodes[1])
    uint32_t next_recv;       // receiver of the edge after the tile (~0: none)
};

// CTAs per SM: three of 256 threads (registers); operand buffers per CTA:
// one with the 144-wide pair input (shared memory), two with the 16-wide
// rows (the next tile's rows are gathered during this tile's layers)
template<bool PAIR>
__host__ __device__ constexpr int
edge_ctas_per_sm()
{
    return 3;
}
template<bool PAIR>
__host__ __device__ constexpr uint32_t
edge_buffers()
{
    return PAIR ? 1u : 2u;
}

template<int K1, bool PAIR, bool SUM>
__global__ void __launch_bounds__(kEdgeThreads, edge_ctas_per_sm<PAIR>())
k_edge_mlp_tc(uint32_t E, const uint16_t* __restrict__ X, uint32_t ldx,
              const uint32_t* __restrict__ recv, const uint32_t* __restrict__ send,
              const uint16_t* __restrict__ H, uint32_t ldh,
              const uint16_t* __restrict__ Ef,
              const uint16_t* __restrict__ W1, const float* __restrict__ b1,
              const uint16_t* __restrict__ W2, const float* __restrict__ b2,
              const uint16_t* __restrict__ W3, const float* __restrict__ b3,
              int act1, int act2, int act3, uint16_t* Y, uint32_t ldy, int* err,
              uint32_t fake,
              uint32_t n_nodes, const uint32_t* __restrict__ off, float scale,
              uint32_t col)
{
    constexpr uint32_t kW1 = ((64u * K1 * 2u + 1023u) / 1024u) * 1024u;
    constexpr uint32_t kW = 64u * 64u * 2u;            // W2, W3
    constexpr uint32_t kOp = edge_operand_bytes<K1>();
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    uint8_t* sW1 = smem;
    uint8_t* sW2 = sW1 + kW1;
    uint8_t* sW3 = sW2 + kW;
    // an operand buffer holds the layer-1 input (128 x K1), then, once
    // layer 1's MMAs have completed, the 128 x 64 activations of layers 1
    // and 2 (and, with SUM, the layer-3 output tile); of the two buffers,
    // the next tile's input is gathered into the other one while this
    // tile's layers run
    constexpr uint32_t kBufs = edge_buffers<PAIR>();
    uint8_t* const sA0 = sW3 + kW;
    uint8_t* sA1 = sA0;  // the current tile's buffer
    EdgeShared* ss = reinterpret_cast<EdgeShared*>(sA0 + kBufs * kOp);
    const uint32_t tid = threadIdx.x;
    const uint32_t warp = tid >> 5, lane = tid & 31;

    for (uint32_t e = tid; e < 64u * K1 / 8u; e += kEdgeThreads) {
        const uint32_t row = e / (K1 / 8), g = e % (K1 / 8);
        *reinterpret_cast<uint4*>(sW1 + ((row / 8) * (K1 / 8) + g) * 128 + (row % 8) * 16) =
            *reinterpret_cast<const uint4*>(W1 + (size_t)row * K1 + g * 8);
    }
    for (uint32_t e = tid; e < 64u * 8u; e += kEdgeThreads) {
        const uint32_t row = e / 8, g = e % 8;
        const uint32_t o = ((row / 8) * 8 + g) * 128 + (row % 8) * 16;
        *reinterpret_cast<uint4*>(sW2 + o) =
            *reinterpret_cast<const uint4*>(W2 + (size_t)row * 64 + g * 8);
        *reinterpret_cast<uint4*>(sW3 + o) =
            *reinterpret_cast<const uint4*>(W3 + (size_t)row * 64 + g * 8);
    }
    if (tid < 192)
        ss->bias[tid / 64][tid % 64] = (tid < 64 ? b1 : (tid < 128 ? b2 : b3))[tid % 64];
    if (tid == 0)
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(smem_addr(&mbar)));
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 "
                     "[%0], %1;\n" :: "r"(smem_addr(&tmem_base)), "r"(64u));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    const uint32_t tmem = tmem_base;
    const uint32_t idesc = make_idesc(64);
    uint32_t phase = 0;
    bool failed = false;

    // issue the MMAs of one layer (thread 0) and wait for them (everyone)
    bool tile_bad = false;
    auto layer = [&](const uint8_t* sA, const uint8_t* sB, uint32_t K) {
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;\n");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n");
            const uint32_t sbo = (K / 8) * 128;
            for (uint32_t ks = 0; ks < K / 16; ks++) {
                const uint64_t ad = make_desc(smem_addr(sA) + ks * 256, 128, sbo);
                const uint64_t bd = make_desc(smem_addr(sB) + ks * 256, 128, sbo);
                const uint32_t acc = ks > 0 ? 1u : 0u;
                asm volatile(
                    "{\n.reg .pred p;\nsetp.ne.u32 p, %4, 0;\n"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                    :: "r"(tmem), "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one."
                         "shared::cluster.b64 [%0];\n" :: "r"(smem_addr(&mbar)));
        }
        uint32_t done = 0;
        for (uint32_t it = 0; it < kWaitLimit && !done; it++) {
            asm volatile("{\n.reg .pred p;\n"
                         "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                         "selp.u32 %0, 1, 0, p;\n}\n"
                         : "=r"(done) : "r"(smem_addr(&mbar)), "r"(phase));
        }
        // a time-out is recorded and acted on at the end of the tile (one
        // CTA-wide vote per tile instead of one per layer)
        const bool bad = !__all_sync(0xffffffffu, done) || fake != 0u;
        if (bad && lane == 0)
            atomicExch(err, 1);
        tile_bad = tile_bad || bad;
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;\n");
    };
    // this thread's row of the accumulator and half of its columns
    const uint32_t row = (warp & 3u) * 32u + lane;
    const uint32_t half = warp >> 2;
    // read the accumulator (32 columns), add the bias, activate;
    // `emit(g, packed8)` receives the row's k-group g (8 bf16 as a uint4)
    auto epilogue = [&](int layer_index, int act, auto&& emit) {
        const uint32_t taddr = tmem + (((warp & 3u) * 32u) << 16) + half * 32u;
        uint32_t v[32];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
            "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]),
              "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]),
              "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
              "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]),
              "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
              "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
              "=r"(v[30]), "=r"(v[31])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;\n");
        const float* bias = ss->bias[layer_index] + half * 32u;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            uint32_t p[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int c = q * 8 + 2 * j;
                const float z0 = __uint_as_float(v[c]) + bias[c];
                const float z1 = __uint_as_float(v[c + 1]) + bias[c + 1];
                p[j] = pack2(z0, z1);
                if (act == AQUA_ACT_SILU)
                    p[j] = silu_bf16x2(p[j]);
            }
            emit((int)(half * 4u) + q, make_uint4(p[0], p[1], p[2], p[3]));
        }
    };
    auto to_a1 = [&](int g, uint4 val) {
        *reinterpret_cast<uint4*>(sA1 + ((row / 8) * 8 + g) * 128 + (row % 8) * 16) = val;
    };

    // the edges of this CTA: every tile (grid-stride), or, with SUM, the
    // edges of its receivers
    uint32_t e_begin = 0, e_end = E;
    if constexpr (SUM) {
        if (tid == 0) {
            // first node s in [0, n_nodes] with off[s] >= v
            auto lower = [&](uint64_t v) -> uint32_t {
                uint32_t lo = 0, hi = n_nodes;
                while (lo < hi) {
                    const uint32_t mid = lo + (hi - lo) / 2;
                    if ((uint64_t)off[mid] < v)
                        lo = mid + 1;
                    else
                        hi = mid;
                }
                return lo;
            };
            const uint64_t G = gridDim.x;
            ss->nodes[0] = blockIdx.x == 0 ? 0u : lower((uint64_t)blockIdx.x * E / G);
            ss->nodes[1] = blockIdx.x + 1 == gridDim.x
                               ? n_nodes
                               : lower((uint64_t)(blockIdx.x + 1) * E / G);
            ss->carry_node[0] = ss->carry_node[1] = 0xffffffffu;
        }
        __syncthreads();
        const uint32_t n_lo = ss->nodes[0], n_hi = ss->nodes[1];
        // receivers without edges: a zero sum
        for (uint32_t s = n_lo + tid; s < n_hi; s += kEdgeThreads)
            if (off[s] == off[s + 1]) {
                uint4* dst = reinterpret_cast<uint4*>(Y + (size_t)s * ldy + col);
                for (int g = 0; g < 8; g++)
                    dst[g] = make_uint4(0u, 0u, 0u, 0u);
            }
        e_begin = off[n_lo];
        e_end = off[n_hi];
    }
    const uint32_t tiles = SUM ? (e_end - e_begin + kTcRows - 1) / kTcRows
                               : (E + kTcRows - 1) / kTcRows;
    // the edge indices of tile t's rows, loaded one tile ahead: the
    // receiver (threads of the first part; ~0 past the last edge) and the
    // sender (pair input)
    constexpr uint32_t kg = K1 / 8;
    const uint32_t grow = tid % kTcRows, part = tid / kTcRows;
    auto load_idx = [&](uint32_t t, uint32_t& ei, uint32_t& es) {
        ei = 0xffffffffu;
        es = 0u;
        if (t >= tiles)
            return;
        const uint32_t e = e_begin + t * kTcRows + grow;
        if (e >= e_end)
            return;
        if ((PAIR || SUM) && part == 0)
            ei = recv[e];
        if (PAIR)
            es = send[e];
    };
    // gathers the layer-1 input of tile t into buf: thread t copies k-groups
    // [part * kg / 2, (part + 1) * kg / 2) of row t % 128 (asynchronous
    // copies, committed by the caller)
    auto gather = [&](uint32_t t, uint8_t* buf, uint32_t ei, uint32_t es) {
        const uint32_t e = e_begin + t * kTcRows + grow;
        const bool valid = e < e_end;
        uint8_t* row0 = buf + (grow / 8) * kg * 128 + (grow % 8) * 16;
        const uint32_t g0 = part * (kg / 2), g1 = g0 + kg / 2;
        if (PAIR) {
            const uint32_t eiv = (valid && part == 0) ? ei : 0u;
            const uint32_t esv = valid ? es : 0u;
            for (uint32_t g = g0; g < g1; g++) {
                const uint16_t* src =
                    g < 8 ? H + (size_t)eiv * ldh + g * 8
                          : (g < 16 ? H + (size_t)esv * ldh + (g - 8) * 8
                                    : Ef + (size_t)(valid ? e : 0u) * 16 + (g - 16) * 8);
                cp_async_16z(row0 + g * 128, src, valid);
            }
        } else {
            for (uint32_t g = g0; g < g1; g++)
                cp_async_16z(row0 + g * 128, X + (size_t)(valid ? e : 0u) * ldx + g * 8,
                             valid);
        }
    };
    const uint32_t stride = SUM ? 1u : gridDim.x;
    uint32_t tile = SUM ? 0u : blockIdx.x;
    uint32_t ei_cur, es_cur;
    load_idx(tile, ei_cur, es_cur);
    uint32_t cur = 0;
    if (kBufs == 2 && tile < tiles)
        gather(tile, sA0, ei_cur, es_cur);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    for (; tile < tiles && !failed; tile += stride) {
        const uint32_t next = tile + stride;
        uint32_t ei_next, es_next;
        load_idx(next, ei_next, es_next);
        if constexpr (kBufs == 2) {
            // the next tile's gather overlaps this tile's layers
            if (next < tiles)
                gather(next, sA0 + (cur ^ 1u) * kOp, ei_next, es_next);
            asm volatile("cp.async.commit_group;\n" ::: "memory");
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        } else {
            gather(tile, sA0, ei_cur, es_cur);
            asm volatile("cp.async.commit_group;\n" ::: "memory");
            asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        }
        const uint32_t eb = e_begin + tile * kTcRows;
        const uint32_t e = eb + row;
        const bool valid = e < e_end;
        sA1 = sA0 + cur * kOp;
        if (SUM && part == 0)
            ss->recv[grow] = ei_cur;
        // the receiver of the edge after this tile's (~0 at the end of the
        // CTA's edges): it tells whether the tile's last run is complete
        if (SUM && tid == 0)
            ss->next_recv = ei_next;
        layer(sA1, sW1, K1);
        epilogue(0, act1, to_a1);
        layer(sA1, sW2, 64);
        epilogue(1, act2, to_a1);
        layer(sA1, sW3, 64);
        if constexpr (!SUM) {
            epilogue(2, act3, [&](int g, uint4 val) {
                if (valid)
                    *reinterpret_cast<uint4*>(Y + (size_t)e * ldy + g * 8) = val;
            });
        } else {
            // layer-3 tile into shared memory: row r at r * 128 bytes, its
            // 16-byte group g at position g ^ (r % 8)
            epilogue(2, act3, [&](int g, uint4 val) {
                *reinterpret_cast<uint4*>(sA1 + row * 128u + ((g ^ (row & 7u)) * 16u)) = val;
            });
            const uint32_t nvalid = min((uint32_t)kTcRows, e_end - eb);
            if (warp < 4) {
                const uint32_t rr = warp * 32u + lane;
                const bool st = rr < nvalid && (rr == 0 || ss->recv[rr] != ss->recv[rr - 1]);
                const uint32_t bal = __ballot_sync(0xffffffffu, st);
                if (lane == 0)
                    ss->start[warp] = bal;
            }
            __syncthreads();
            const uint32_t par = tile & 1u;
            uint32_t ord = 0;
            for (uint32_t wq = 0; wq < 4; wq++) {
                uint32_t m = ss->start[wq];
                while (m) {
                    const uint32_t a = wq * 32u + (uint32_t)(__ffs(m) - 1);
                    m &= m - 1;
                    if ((ord++ % kEdgeWarps) != warp)
                        continue;
                    // the run ends at the next start or at the last row
                    uint32_t b = nvalid;
                    if (m) {
                        b = wq * 32u + (uint32_t)(__ffs(m) - 1);
                    } else {
                        for (uint32_t w2 = wq + 1; w2 < 4; w2++) {
                            const uint32_t m2 = ss->start[w2];
                            if (m2) {
                                b = w2 * 32u + (uint32_t)(__ffs(m2) - 1);
                                break;
                            }
                        }
                    }
                    const uint32_t node = ss->recv[a];
                    float a0 = 0.f, a1 = 0.f;
                    if (a == 0 && ss->carry_node[par] == node) {
                        a0 = ss->carry[par][2 * lane];
                        a1 = ss->carry[par][2 * lane + 1];
                    }
                    // row k's two columns of this lane
                    auto ld_row = [&](uint32_t k) -> uint32_t {
                        return *reinterpret_cast<const uint32_t*>(
                            sA1 + k * 128u + (((lane >> 2) ^ (k & 7u)) * 16u) +
                            (lane & 3u) * 4u);
                    };
                    // eight loads in flight, then the additions in row order
                    uint32_t k = a;
                    for (; k + 8u <= b; k += 8u) {
                        uint32_t v[8];
#pragma unroll
                        for (int u = 0; u < 8; u++)
                            v[u] = ld_row(k + u);
#pragma unroll
                        for (int u = 0; u < 8; u++) {
                            a0 += __uint_as_float(v[u] << 16);
                            a1 += __uint_as_float(v[u] & 0xffff0000u);
                        }
                    }
                    for (; k < b; k++) {
                        const uint32_t v = ld_row(k);
                        a0 += __uint_as_float(v << 16);
                        a1 += __uint_as_float(v & 0xffff0000u);
                    }
                    if (b < nvalid || ss->next_recv != node) {
                        *reinterpret_cast<uint32_t*>(Y + (size_t)node * ldy + col +
                                                     2 * lane) =
                            pack2(a0 * scale, a1 * scale);
                    } else {
                        // the last run: its receiver continues in the next tile
                        ss->carry[par ^ 1u][2 * lane] = a0;
                        ss->carry[par ^ 1u][2 * lane + 1] = a1;
                        if (lane == 0)
                            ss->carry_node[par ^ 1u] = node;
                    }
                }
            }
        }
        // the tile after next reuses this buffer; the next tile's MMAs
        // reuse the accumulator; a time-out in any layer ends the CTA
        asm volatile("tcgen05.fence::before_thread_sync;\n");
        failed = __syncthreads_or(tile_bad);
        ei_cur = ei_next;
        es_cur = es_next;
        cur = (cur + 1u) % kBufs;
    }
    // no copy may still be in flight when the CTA ends (after a time-out)
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n"
                     :: "r"(tmem), "r"(64u));
    }
}

template<int K1>
constexpr size_t
edge_mlp_smem()
{
    return ((64u * K1 * 2u + 1023u) / 1024u) * 1024u + 2u * 64u * 64u * 2u +
           edge_buffers<K1 == 144>() * edge_operand_bytes<K1>() + sizeof(EdgeShared);
}
static_assert(edge_ctas_per_sm<true>() * (edge_mlp_smem<144>() + 1024) <= 228 * 1024,
              "pair-input CTAs per SM");
static_assert(edge_ctas_per_sm<false>() * (edge_mlp_smem<16>() + 1024) <= 228 * 1024,
              "row-input CTAs per SM");
static_assert(edge_ctas_per_sm<false>() * (edge_mlp_smem<80>() + 1024) <= 228 * 1024,
              "80-wide row-input CTAs per SM");


// ---------------------------------------------------------------------------
// Backward of a dense layer on the tensor cores (training).
//
// dgrad: dX = dY W, times silu'(Zprev) when the previous layer is SiLU.  It
// is the forward's product with dY (M x N) as A and W^T (K x N, the
// transposed weights kept by the model) as B: reduction over N (16 or 64),
// K output columns (up to 160) in a tensor-memory accumulator of `tcols`
// columns; the epilogue multiplies by silu'(Zprev) and rounds to BF16.
//
// wgrad: dW += dY^T X and db += column sums of dY.  The reduction runs over
// the M rows (edges or nodes), 128 per chunk: each chunk of dY and X is
// staged transposed (dY^T: N rows of 128, padded with zero rows to the
// MMA's 128; X^T: K rows of 128) into the K-major core-matrix layout, and
// the MMAs accumulate over all the CTA's chunks in tensor memory.  One
// extra row of ones in B makes the column K of the product the column sums
// of dY (db).  At the end each CTA adds its partial dW, db to the outputs
// with atomics.

__device__ __forceinline__ float
silu_grad_f(float z)
{
    const float s = 1.f / (1.f + __expf(-z));
    return s * (1.f + z * (1.f - s));
}

// bounded wait for a commit on `mbar` (phase parity `phase`); every thread
// of the CTA returns the same verdict
__device__ __forceinline__ bool
tc_wait(uint64_t* mbar, uint32_t phase, uint32_t fake)
{
    uint32_t done = 0;
    for (uint32_t it = 0; it < kWaitLimit && !done; it++) {
        asm volatile("{\n.reg .pred p;\n"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                     "selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(done) : "r"(smem_addr(mbar)), "r"(phase));
    }
    // `fake` (test switch): a wait that completed counts as timed out
    return !__syncthreads_or(!done || fake);
}

__global__ void __launch_bounds__(kTcThreads, 1)
k_linear_dgrad_tc(uint32_t M, uint32_t N, uint32_t K,
                  const uint16_t* __restrict__ dY, uint32_t ldy,
                  const uint16_t* __restrict__ Wt,
                  const float* __restrict__ Zp, uint32_t ldzp, int act_prev,
                  uint16_t* dX, uint32_t ldx, uint32_t tcols, int* err,
                  uint32_t fake)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    uint8_t* sB = smem;                                        // K x N
    uint8_t* sA = smem + ((K * N * 2 + 1023) / 1024) * 1024;   // 128 x N
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    stage(sB, Wt, N, K, K, N);
    if (threadIdx.x == 0)
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n"
                     :: "r"(smem_addr(&mbar)));
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 "
                     "[%0], %1;\n" :: "r"(smem_addr(&tmem_base)), "r"(tcols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    const uint32_t tmem = tmem_base;
    const uint32_t idesc = make_idesc(K);
    const uint32_t sbo = (N / 8) * 128;
    uint32_t phase = 0;
    const uint32_t tiles = (M + kTcRows - 1) / kTcRows;
    for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const uint32_t m0 = tile * kTcRows;
        const uint32_t valid = min((uint32_t)kTcRows, M - m0);
        stage(sA, dY + (size_t)m0 * ldy, ldy, kTcRows, valid, N);
        asm volatile("fence.proxy.async.shared::cta;\n");
        __syncthreads();
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n");
            for (uint32_t ks = 0; ks < N / 16; ks++) {
                const uint64_t ad = make_desc(smem_addr(sA) + ks * 256, 128, sbo);
                const uint64_t bd = make_desc(smem_addr(sB) + ks * 256, 128, sbo);
                const uint32_t acc = ks > 0 ? 1u : 0u;
                asm volatile(
                    "{\n.reg .pred p;\nsetp.ne.u32 p, %4, 0;\n"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                    :: "r"(tmem), "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one."
                         "shared::cluster.b64 [%0];\n" :: "r"(smem_addr(&mbar)));
        }
        if (!tc_wait(&mbar, phase, fake)) {
            if (threadIdx.x == 0)
                atomicExch(err, 1);
            tc_wait(&mbar, phase, 0u);  // the MMAs in flight, again bounded
            break;
        }
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;\n");
        // epilogue: warp w owns rows 32w .. 32w + 31 (TMEM lanes)
        const uint32_t row = m0 + warp * 32 + lane;
        const uint32_t taddr = tmem + ((warp * 32u) << 16);
        for (uint32_t c0 = 0; c0 < K; c0 += 16) {
            uint32_t v[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]),
                  "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]),
                  "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                  "=r"(v[14]), "=r"(v[15])
                : "r"(taddr + c0));
            asm volatile("tcgen05.wait::ld.sync.aligned;\n");
            if (row < M) {
                float d[16];
                for (int j = 0; j < 16; j++)
                    d[j] = __uint_as_float(v[j]);
                if (Zp && act_prev == AQUA_ACT_SILU) {
                    const float* z = Zp + (size_t)row * ldzp + c0;
                    for (int j = 0; j < 16; j += 4) {
                        const float4 zz = *reinterpret_cast<const float4*>(z + j);
                        d[j] *= silu_grad_f(zz.x);
                        d[j + 1] *= silu_grad_f(zz.y);
                        d[j + 2] *= silu_grad_f(zz.z);
                        d[j + 3] *= silu_grad_f(zz.w);
                    }
                }
                uint32_t pk[8];
                for (int j = 0; j < 8; j++)
                    pk[j] = pack2(d[2 * j], d[2 * j + 1]);
                uint4* dst = reinterpret_cast<uint4*>(dX + (size_t)row * ldx + c0);
                dst[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                dst[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
            }
        }
        // the next tile's MMAs overwrite the accumulator and sA
        asm volatile("tcgen05.fence::before_thread_sync;\n");
        __syncthreads();
    }
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n"
                     :: "r"(tmem), "r"(tcols));
    }
}

// rows x 128 transposed block: element (r, m) = src[m * ld + r] for r < nr
// and m < valid (zero for m >= valid), into the core-matrix layout with 128
// reduction columns (16 core matrices per 8-row group); rows >= nr are left
// as they are.  Each warp task moves four 8 x 8 blocks (four consecutive
// 8-row groups of m, one 8-column group of r): every lane loads its
// fragment element pair from global memory (row m = lane / 4, columns
// 2 (lane % 4) and the next) and stmatrix .trans writes each block
// transposed, whole 16-byte rows of a core matrix, free of bank conflicts.
__device__ __forceinline__ void
stage_t(uint8_t* dst, const uint16_t* src, uint32_t ld, uint32_t nr,
        uint32_t valid)
{
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t rg = nr / 8;                        // 8-column groups of r
    const uint32_t ar = lane >> 2, ac = (lane & 3) * 2;  // fragment position
    const uint32_t mi = lane >> 3, mj = lane & 7;        // row address role
    for (uint32_t t = warp; t < 4 * rg; t += blockDim.x / 32) {
        const uint32_t mg = t & 3, kb = t >> 2;
        uint32_t v[4];
        for (int i = 0; i < 4; i++) {
            const uint32_t m = (mg * 4 + i) * 8 + ar;
            v[i] = m < valid ? *reinterpret_cast<const uint32_t*>(
                                   src + (size_t)m * ld + kb * 8 + ac)
                             : 0u;
        }
        // lane 8i + j: row j of block i, stored transposed at the core
        // matrix (r group kb, m group 4 mg + i)
        const uint32_t addr =
            smem_addr(dst + (kb * 16 + mg * 4 + mi) * 128 + mj * 16);
        asm volatile("stmatrix.sync.aligned.m8n8.x4.trans.shared.b16 "
                     "[%0], {%1, %2, %3, %4};\n"
                     :: "r"(addr), "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3])
                     : "memory");
    }
}

constexpr int kWgThreads = 256;  // wgrad: 8 warps stage, warps 0-3 read TMEM

__global__ void __launch_bounds__(kWgThreads, 1)
k_linear_wgrad_tc(uint32_t M, uint32_t N, uint32_t K,
                  const uint16_t* __restrict__ dY, uint32_t ldy,
                  const uint16_t* __restrict__ X, uint32_t ldx, float* dW,
                  float* db, uint32_t KB, uint32_t nbuf, uint32_t tcols,
                  int* err, uint32_t fake)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_base;
    // nbuf (1 or 2) buffers, each A = dY^T (128 rows, N used) x 128 and
    // B = X^T (KB rows: X^T, then the row of ones for db, then zeros) x 128;
    // with two, a chunk is staged while the MMAs of the previous one run
    const uint32_t bufb = 128 * 128 * 2 + KB * 128 * 2;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t chunks = (M + kTcRows - 1) / kTcRows;
    if ((uint32_t)blockIdx.x >= chunks)
        return;  // no chunk for this CTA (before any allocation)
    for (uint32_t b = 0; b < nbuf; b++) {
        uint8_t* sA = smem + b * bufb;
        uint8_t* sB = sA + 128 * 128 * 2;
        for (uint32_t e = threadIdx.x; e < 128u * 128u / 8u; e += kWgThreads)
            reinterpret_cast<uint4*>(sA)[e] = make_uint4(0, 0, 0, 0);
        for (uint32_t e = threadIdx.x; e < (KB - K) * 128u; e += kWgThreads) {
            const uint32_t r = K + e / 128u, m = e % 128u;
            const uint16_t one = (r == K && db) ? 0x3F80u : 0u;  // bf16 1.0
            *reinterpret_cast<uint16_t*>(
                sB + ((r / 8) * 16 + m / 8) * 128 + (r % 8) * 16 + (m % 8) * 2) = one;
        }
    }
    if (threadIdx.x == 0)
        for (int b = 0; b < 2; b++)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n"
                         :: "r"(smem_addr(&mbar[b])));
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 "
                     "[%0], %1;\n" :: "r"(smem_addr(&tmem_base)), "r"(tcols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    const uint32_t tmem = tmem_base;
    const uint32_t idesc = make_idesc(KB);
    constexpr uint32_t sbo = 16 * 128;  // 128 reduction columns per row group
    uint32_t phase[2] = { 0u, 0u };
    uint32_t pending[2] = { 0u, 0u };  // a commit of the buffer not yet waited
    bool failed = false;
    uint32_t it = 0;
    for (uint32_t ch = blockIdx.x; ch < chunks && !failed; ch += gridDim.x, it++) {
        const uint32_t b = it % nbuf;
        uint8_t* sA = smem + b * bufb;
        uint8_t* sB = sA + 128 * 128 * 2;
        // the MMAs of the chunk nbuf ago read this buffer
        if (pending[b]) {
            if (!tc_wait(&mbar[b], phase[b], fake)) {
                failed = true;
                break;
            }
            phase[b] ^= 1u;
            pending[b] = 0u;
        }
        const uint32_t m0 = ch * kTcRows;
        const uint32_t valid = min((uint32_t)kTcRows, M - m0);
        stage_t(sA, dY + (size_t)m0 * ldy, ldy, N, valid);
        stage_t(sB, X + (size_t)m0 * ldx, ldx, K, valid);
        asm volatile("fence.proxy.async.shared::cta;\n");
        __syncthreads();
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n");
            for (uint32_t ks = 0; ks < 8; ks++) {
                const uint64_t ad = make_desc(smem_addr(sA) + ks * 256, 128, sbo);
                const uint64_t bd = make_desc(smem_addr(sB) + ks * 256, 128, sbo);
                const uint32_t acc = (it == 0 && ks == 0) ? 0u : 1u;
                asm volatile(
                    "{\n.reg .pred p;\nsetp.ne.u32 p, %4, 0;\n"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                    :: "r"(tmem), "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one."
                         "shared::cluster.b64 [%0];\n" :: "r"(smem_addr(&mbar[b])));
        }
        pending[b] = 1u;
    }
    // the last commits (the MMAs run in order: the later one covers both)
    for (int b = 0; b < 2; b++) {
        if (!pending[b])
            continue;
        if (!tc_wait(&mbar[b], phase[b], failed ? 0u : fake)) {
            failed = true;
            tc_wait(&mbar[b], phase[b], 0u);  // in flight, again bounded
        }
    }
    if (failed) {
        if (threadIdx.x == 0)
            atomicExch(err, 1);
    } else if (warp < 4) {
        asm volatile("tcgen05.fence::after_thread_sync;\n");
        // epilogue: rows n = 32w + lane < N add their partial sums
        const uint32_t n = warp * 32 + lane;
        const uint32_t taddr = tmem + ((warp * 32u) << 16);
        for (uint32_t c0 = 0; c0 < KB; c0 += 16) {
            uint32_t v[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]),
                  "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]),
                  "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                  "=r"(v[14]), "=r"(v[15])
                : "r"(taddr + c0));
            asm volatile("tcgen05.wait::ld.sync.aligned;\n");
            if (n < N) {
                for (int j = 0; j < 16; j++) {
                    const uint32_t col = c0 + j;
                    if (col < K)
                        atomicAdd(&dW[(size_t)n * K + col], __uint_as_float(v[j]));
                    else if (col == K && db)
                        atomicAdd(&db[n], __uint_as_float(v[j]));
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n"
                     :: "r"(tmem), "r"(tcols));
    }
}
}  // namespace

namespace {

// sets the shared-memory limit of the four fused edge-MLP kernels once per
// device (the limit is a per-device attribute of each kernel)
aqua_status
edge_mlp_configure(int& sms)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
            cudaSuccess)
        return AQUA_ERR_CUDA;
    static std::atomic<uint64_t> configured{ 0 };
    const uint64_t bit = dev < 64 ? (1ull << dev) : 0ull;
    if (!bit || !(configured.load() & bit)) {
        const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
        if (cudaFuncSetAttribute(k_edge_mlp_tc<16, false, false>, a,
                                 (int)edge_mlp_smem<16>()) != cudaSuccess ||
            cudaFuncSetAttribute(k_edge_mlp_tc<80, false, false>, a,
                                 (int)edge_mlp_smem<80>()) != cudaSuccess ||
            cudaFuncSetAttribute(k_edge_mlp_tc<144, true, false>, a,
                                 (int)edge_mlp_smem<144>()) != cudaSuccess ||
            cudaFuncSetAttribute(k_edge_mlp_tc<16, false, true>, a,
                                 (int)edge_mlp_smem<16>()) != cudaSuccess ||
            cudaFuncSetAttribute(k_edge_mlp_tc<144, true, true>, a,
                                 (int)edge_mlp_smem<144>()) != cudaSuccess)
            return AQUA_ERR_CUDA;
        configured.fetch_or(bit);
    }
    return AQUA_OK;
}

bool
a16(const void* p)
{
    return (reinterpret_cast<uintptr_t>(p) & 15) == 0;
}

// the arguments both fused forms share; row inputs are 16 wide (edge
// features), or 80 wide where `rows80` (the first node MLP, n1)
bool
edge_mlp_args_ok(uint32_t K1, bool rows80, const uint16_t* X, uint32_t ldx,
                 const uint32_t* recv, const uint32_t* send, const uint16_t* H,
                 uint32_t ldh, const uint16_t* Ef, const uint16_t* W1,
                 const float* b1, const uint16_t* W2, const float* b2,
                 const uint16_t* W3, const float* b3, const int32_t* err)
{
    if (!W1 || !b1 || !W2 || !b2 || !W3 || !b3 || !err || !a16(W1) ||
        !a16(W2) || !a16(W3))
        return false;
    if (X == nullptr)
        return K1 == 144 && recv && send && H && Ef && ldh >= 64 && ldh % 8 == 0 &&
               a16(H) && a16(Ef);
    return (K1 == AQUA_GNN_FEATURES || (rows80 && K1 == 80)) && ldx >= K1 &&
           ldx % 8 == 0 && a16(X);
}

}  // namespace

extern "C" aqua_status
aqua_gnn_edge_mlp_tc(uint32_t E, uint32_t K1, const uint16_t* X, uint32_t ldx,
                     const uint32_t* recv, const uint32_t* send,
                     const uint16_t* H, uint32_t ldh, const uint16_t* Ef,
                     const uint16_t* W1, const float* b1, const uint16_t* W2,
                     const float* b2, const uint16_t* W3, const float* b3,
                     int32_t act1, int32_t act2, int32_t act3, uint16_t* Y,
                     uint32_t ldy, int32_t* err, void* stream)
{
    const bool pair = (X == nullptr);
    if (!edge_mlp_args_ok(K1, true, X, ldx, recv, send, H, ldh, Ef, W1, b1, W2,
                          b2, W3, b3, err) ||
        !Y || ldy < 64 || ldy % 8 || !a16(Y))
        return AQUA_ERR_INVALID;
    if (E == 0)
        return AQUA_OK;
    int sms = 0;
    const aqua_status st = edge_mlp_configure(sms);
    if (st != AQUA_OK)
        return st;
    const uint32_t tiles = (E + kTcRows - 1) / kTcRows;
    cudaStream_t s = (cudaStream_t)stream;
    if (pair) {
        // 72 KB of shared memory: three CTAs per SM (192 of 512 TMEM columns)
        const uint32_t cap = (uint32_t)sms * edge_ctas_per_sm<true>();
        const uint32_t grid = tiles < cap ? tiles : cap;
        k_edge_mlp_tc<144, true, false>
            <<<grid, kEdgeThreads, edge_mlp_smem<144>(), s>>>(
                E, nullptr, 0, recv, send, H, ldh, Ef, W1, b1, W2, b2, W3, b3,
                act1, act2, act3, Y, ldy, err, (uint32_t)aqua::g_debug_fake_timeout, 0u, nullptr, 0.f, 0u);
    } else if (K1 == 80) {
        // the first node MLP, n1 (80-wide rows): 70 KB, three CTAs per SM
        const uint32_t cap = (uint32_t)sms * edge_ctas_per_sm<false>();
        const uint32_t grid = tiles < cap ? tiles : cap;
        k_edge_mlp_tc<80, false, false>
            <<<grid, kEdgeThreads, edge_mlp_smem<80>(), s>>>(
                E, X, ldx, nullptr, nullptr, nullptr, 0, nullptr, W1, b1, W2,
                b2, W3, b3, act1, act2, act3, Y, ldy, err, (uint32_t)aqua::g_debug_fake_timeout, 0u, nullptr, 0.f, 0u);
    } else {
        // 52 KB: three CTAs per SM (registers; 192 TMEM columns)
        const uint32_t cap = (uint32_t)sms * edge_ctas_per_sm<false>();
        const uint32_t grid = tiles < cap ? tiles : cap;
        k_edge_mlp_tc<16, false, false>
            <<<grid, kEdgeThreads, edge_mlp_smem<16>(), s>>>(
                E, X, ldx, nullptr, nullptr, nullptr, 0, nullptr, W1, b1, W2,
                b2, W3, b3, act1, act2, act3, Y, ldy, err, (uint32_t)aqua::g_debug_fake_timeout, 0u, nullptr, 0.f, 0u);
    }
    return cudaGetLastError() == cudaSuccess ? AQUA_OK : AQUA_ERR_CUDA;
}

extern "C" aqua_status
aqua_gnn_edge_mlp_sum_tc(uint32_t n_nodes, uint32_t E, uint32_t K1,
                         const uint16_t* X, uint32_t ldx,
                         const uint32_t* offsets, const uint32_t* recv,
                         const uint32_t* send, const uint16_t* H, uint32_t ldh,
                         const uint16_t* Ef, const uint16_t* W1,
                         const float* b1, const uint16_t* W2, const float* b2,
                         const uint16_t* W3, const float* b3, int32_t act1,
                         int32_t act2, int32_t act3, float scale,
                         uint16_t* out, uint32_t ld, uint32_t col,
                         int32_t* err, void* stream)
{
    const bool pair = (X == nullptr);
    if (!edge_mlp_args_ok(K1, false, X, ldx, recv, send, H, ldh, Ef, W1, b1, W2, b2,
                          W3, b3, err) ||
        !offsets || !recv || !out || !a16(out) || ld % 8 || col % 8 ||
        col + 64 > ld || E >= 0x80000000u)
        return AQUA_ERR_INVALID;
    if (n_nodes == 0)
        return AQUA_OK;
    int sms = 0;
    const aqua_status st = edge_mlp_configure(sms);
    if (st != AQUA_OK)
        return st;
    // each CTA owns the receivers of about E / grid edges; a small graph
    // gets fewer CTAs (at least one, for the receivers without edges)
    const uint32_t tiles = (E + kTcRows - 1) / kTcRows;
    const uint32_t per_sm = (uint32_t)(pair ? edge_ctas_per_sm<true>()
                                             : edge_ctas_per_sm<false>());
    uint32_t grid = (uint32_t)sms * per_sm;
    if (tiles < grid)
        grid = tiles > 0 ? tiles : 1u;
    cudaStream_t s = (cudaStream_t)stream;
    if (pair)
        k_edge_mlp_tc<144, true, true>
            <<<grid, kEdgeThreads, edge_mlp_smem<144>(), s>>>(
                E, nullptr, 0, recv, send, H, ldh, Ef, W1, b1, W2, b2, W3, b3,
                act1, act2, act3, out, ld, err, (uint32_t)aqua::g_debug_fake_timeout, n_nodes, offsets, scale, col);
    else
        k_edge_mlp_tc<16, false, true>
            <<<grid, kEdgeThreads, edge_mlp_smem<16>(), s>>>(
                E, X, ldx, recv, nullptr, nullptr, 0, nullptr, W1, b1, W2, b2,
                W3, b3, act1, act2, act3, out, ld, err, (uint32_t)aqua::g_debug_fake_timeout, n_nodes, offsets, scale,
                col);
    return cudaGetLastError() == cudaSuccess ? AQUA_OK : AQUA_ERR_CUDA;
}

extern "C" aqua_status
aqua_gnn_linear_fwd_tc(uint32_t M, uint32_t K, uint32_t N, const uint16_t* X,
                       uint32_t ldx, const uint16_t* W, const float* b,
                       float* Z, uint32_t ldz, uint16_t* Y, uint32_t ldy,
                       int32_t act, int32_t* err, void* stream)
{
    if (!X || !W || !err || (!Z && !Y) || K == 0 || K % 16 || K > 160 ||
        N != 64 || ldx < K || ldx % 8 || (Z && (ldz < N || ldz % 4)) ||
        (Y && (ldy < N || ldy % 8)) ||
        (reinterpret_cast<uintptr_t>(X) & 15) || (reinterpret_cast<uintptr_t>(W) & 15) ||
        (Z && (reinterpret_cast<uintptr_t>(Z) & 15)) ||
        (Y && (reinterpret_cast<uintptr_t>(Y) & 15)))
        return AQUA_ERR_INVALID;
    if (M == 0)
        return AQUA_OK;
    size_t bytes = ((size_t)N * K * 2 + 1023) / 1024 * 1024 +
                   (size_t)kTcRows * K * 2;
    // at least 30 KB per CTA keeps <= 7 CTAs on an SM (7 x 64 of the 512
    // tensor-memory columns), so tcgen05.alloc never has to wait
    if (bytes < 30 * 1024)
        bytes = 30 * 1024;
    int sms = 0, dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
            cudaSuccess)
        return AQUA_ERR_CUDA;
    static std::atomic<uint64_t> configured{ 0 };
    const uint64_t bit = dev < 64 ? (1ull << dev) : 0ull;
    if (!bit || !(configured.load() & bit)) {
        if (cudaFuncSetAttribute(k_linear_fwd_tc<64>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 64 * 1024) != cudaSuccess)
            return AQUA_ERR_CUDA;
        configured.fetch_or(bit);
    }
    const uint32_t tiles = (M + kTcRows - 1) / kTcRows;
    const uint32_t grid = tiles < (uint32_t)sms * 8u ? tiles : (uint32_t)sms * 8u;
    k_linear_fwd_tc<64><<<grid, kTcThreads, bytes, (cudaStream_t)stream>>>(
        M, K, X, ldx, W, b, Z, ldz, Y, ldy, act, err, (uint32_t)aqua::g_debug_fake_timeout);
    return cudaGetLastError() == cudaSuccess ? AQUA_OK : AQUA_ERR_CUDA;
}

namespace {

// tensor-memory columns for an accumulator of `cols` columns (a power of 2,
// at least 32), and the shared memory that keeps the CTAs of one SM within
// its 512 columns, so that tcgen05.alloc never waits
uint32_t
tc_cols(uint32_t cols)
{
    uint32_t t = 32;
    while (t < cols)
        t *= 2;
    return t;
}

size_t
tc_min_smem(uint32_t tcols)
{
    return (size_t)233472 / (512u / tcols + 1u);
}

cudaError_t
tc_sms(int* sms)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, dev);
    return e;
}

bool
al16(const void* p)
{
    return (reinterpret_cast<uintptr_t>(p) & 15) == 0;
}

}  // namespace

extern "C" aqua_status
aqua_gnn_linear_dgrad_tc(uint32_t M, uint32_t N, uint32_t K,
                         const uint16_t* dY, uint32_t ldy, const uint16_t* Wt,
                         const float* Zprev, uint32_t ldzp, int32_t act_prev,
                         uint16_t* dX, uint32_t ldx, int32_t* err, void* stream)
{
    if (!dY || !Wt || !dX || !err || (N != 16 && N != 64) || K == 0 ||
        K % 16 || K > 160 || ldy < N || ldy % 8 || ldx < K || ldx % 8 ||
        !al16(dY) || !al16(Wt) || !al16(dX) ||
        (Zprev && act_prev == AQUA_ACT_SILU &&
         (ldzp < K || ldzp % 4 || !al16(Zprev))))
        return AQUA_ERR_INVALID;
    if (M == 0)
        return AQUA_OK;
    const uint32_t tcols = tc_cols(K);
    size_t bytes = ((size_t)K * N * 2 + 1023) / 1024 * 1024 + (size_t)kTcRows * N * 2;
    if (bytes < tc_min_smem(tcols))
        bytes = tc_min_smem(tcols);
    int sms = 0;
    if (tc_sms(&sms) != cudaSuccess)
        return AQUA_ERR_CUDA;
    if (cudaFuncSetAttribute(k_linear_dgrad_tc,
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)bytes) != cudaSuccess)
        return AQUA_ERR_CUDA;
    const uint32_t tiles = (M + kTcRows - 1) / kTcRows;
    const uint32_t cap = (uint32_t)sms * (512u / tcols);
    const uint32_t grid = tiles < cap ? tiles : cap;
    k_linear_dgrad_tc<<<grid, kTcThreads, bytes, (cudaStream_t)stream>>>(
        M, N, K, dY, ldy, Wt, Zprev, ldzp, act_prev, dX, ldx, tcols, err,
        (uint32_t)aqua::g_debug_fake_timeout);
    return cudaGetLastError() == cudaSuccess ? AQUA_OK : AQUA_ERR_CUDA;
}

extern "C" aqua_status
aqua_gnn_linear_wgrad_tc(uint32_t M, uint32_t N, uint32_t K,
                         const uint16_t* dY, uint32_t ldy, const uint16_t* X,
                         uint32_t ldx, float* dW, float* db, int32_t* err,
                         void* stream)
{
    if (!dY || !X || !dW || !err || (N != 16 && N != 64) || K == 0 ||
        K % 16 || K > 160 || ldy < N || ldy % 8 || ldx < K || ldx % 8 ||
        !al16(dY) || !al16(X))
        return AQUA_ERR_INVALID;
    if (M == 0)
        return AQUA_OK;
    const uint32_t KB = K + 16;  // + the row of ones (db) and zero padding
    const uint32_t tcols = tc_cols(KB);
    const size_t buf = (size_t)128 * 128 * 2 + (size_t)KB * 128 * 2;
    // two staging buffers where two CTAs per SM still fit, else one
    const uint32_t nbuf = 233472 / (2 * buf + 1024) >= 2 ? 2u : 1u;
    size_t bytes = nbuf * buf;
    if (bytes < tc_min_smem(tcols))
        bytes = tc_min_smem(tcols);
    int sms = 0;
    if (tc_sms(&sms) != cudaSuccess)
        return AQUA_ERR_CUDA;
    if (cudaFuncSetAttribute(k_linear_wgrad_tc,
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)bytes) != cudaSuccess)
        return AQUA_ERR_CUDA;
    const uint32_t chunks = (M + kTcRows - 1) / kTcRows;
    // CTAs resident per SM: tensor-memory columns and shared memory
    uint32_t per_sm = 512u / tcols;
    const uint32_t by_smem = (uint32_t)(233472 / (bytes + 1024));
    if (by_smem < per_sm)
        per_sm = by_smem;
    const uint32_t cap = (uint32_t)sms * (per_sm > 0 ? per_sm : 1u);
    const uint32_t grid = chunks < cap ? chunks : cap;
    k_linear_wgrad_tc<<<grid, kWgThreads, bytes, (cudaStream_t)stream>>>(
        M, N, K, dY, ldy, X, ldx, dW, db, KB, nbuf, tcols, err,
        (uint32_t)aqua::g_debug_fake_timeout);
    return cudaGetLastError() == cudaSuccess ? AQUA_OK : AQUA_ERR_CUDA;
}
