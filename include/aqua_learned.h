/*
 * aqua_learned -- kernels of the learned k-step proposal: a message-passing
 * network over the cell-list neighbour graph of the particles, trained on
 * trajectories of the plain step, that proposes the state k steps ahead.
 *
 * None of these functions has a counterpart in the reference: AQUAgpusph
 * has no learned component.  They live in the same library as the plain
 * step (libaqua_gb300.so) and follow its conventions (include/aqua_gb300.h):
 * extern "C", POD arguments, device pointers, aqua_status returns, a
 * cudaStream_t passed as void*.  Matrices are row-major with an explicit
 * leading dimension in elements; bf16 matrices hold raw 16-bit words
 * (uint16_t); every bf16 leading dimension and every matrix base must be a
 * multiple of 8 elements / 16 bytes.
 *
 * Dense layers run on the tensor cores (BF16 inputs and weights, FP32
 * accumulation).  A layer y = act(x W^T + b) keeps W as N x K (out x in),
 * its transpose Wt as K x N for the data gradient.
 */
#ifndef AQUA_LEARNED_H
#define AQUA_LEARNED_H

#include <stdint.h>

#include "aqua_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

#define AQUA_ACT_NONE 0
#define AQUA_ACT_SILU 1
/* width of the feature rows (node and edge features, zero padded) */
#define AQUA_GNN_FEATURES 16

/* ---- neighbour graph over the particles of a batch of cases ----------- */

/* Cell key of every particle: cases are kept apart by the key
 * (key = cid * cells_per_case + cell), probes (imove == 0) get 0xffffffff.
 * cell coordinates are floor((r - origin) / cell) clamped to [0, ncell).
 * vals = 0 .. n-1.  origin3 and ncell3 are host arrays. */
aqua_status aqua_gnn_cell_keys(uint32_t n, int32_t dims, const float* r,
                               const int32_t* imove, const uint32_t* cid,
                               float cell, const float* origin3,
                               const uint32_t* ncell3, uint32_t* keys,
                               uint32_t* vals, void* stream);
/* cell_start / cell_end of every key (0 / 0 when empty) from the sorted
 * keys; n_keys = cases * cells per case. */
aqua_status aqua_gnn_cell_ranges(uint32_t n, const uint32_t* sorted_keys,
                                 uint32_t n_keys, uint32_t* cell_start,
                                 uint32_t* cell_end, void* stream);
/* Nodes are the particles in sorted-key order (node s = particle perm[s],
 * the first n_nodes sorted keys, probes excluded).  For each node: the
 * nodes of the 3^D cells around it (same case) closer than `radius`,
 * itself excluded, in cell order.  With `senders` NULL only degree[s] is
 * written; otherwise receivers/senders are filled from offsets (exclusive
 * scan of the degrees).  The positions are node-ordered (rs[s]); ncell3 is
 * a host array. */
aqua_status aqua_gnn_neighbours(uint32_t n_nodes, int32_t dims,
                                const float* rs, const uint32_t* sorted_keys,
                                const uint32_t* ncell3,
                                const uint32_t* cell_start,
                                const uint32_t* cell_end, float radius,
                                uint32_t* degree, const uint32_t* offsets,
                                uint32_t* receivers, uint32_t* senders,
                                void* stream);
/* Bounding box of the particles with imove != 0: out (host) = min x, y, z,
 * max x, y, z (z = 0 in 2-D); synchronises.  scratch: 8 device words. */
aqua_status aqua_gnn_bbox(uint32_t n, int32_t dims, const float* r,
                          const int32_t* imove, int32_t* scratch, float* out,
                          void* stream);
/* out[0] = 0, out[i+1] = in[0] + ... + in[i]  (n <= 2^26); scratch holds
 * n / 4096 + 2 words */
aqua_status aqua_gnn_exclusive_scan(uint32_t n, const uint32_t* in,
                                    uint32_t* out, uint32_t* scratch,
                                    void* stream);
/* dst[s * comps + c] = src[perm[s] * src_stride + c] (f32 or 32-bit) */
aqua_status aqua_gnn_gather32(uint32_t n, const uint32_t* perm,
                              const void* src, uint32_t src_stride,
                              uint32_t comps, void* dst, void* stream);
/* dst[perm[s] * dst_stride + c] = src[s * comps + c] */
aqua_status aqua_gnn_scatter32(uint32_t n, const uint32_t* perm,
                               const void* src, uint32_t comps, void* dst,
                               uint32_t dst_stride, void* stream);

/* ---- features ---------------------------------------------------------- */

/* scales[0..5] = h, U (velocity), R (density), A (acceleration),
 * Rd (density rate), rho0.  Node rows (ld elements apart, starting at
 * column `col`): u/U, (rho - rho0)/R, dudt/A, drhodt/Rd, [fluid], [wall],
 * normal (walls); edge rows (16 wide): (r_j - r_i)/h, |r_j - r_i|/h,
 * (u_j - u_i)/U, (rho_j - rho_i)/R, Wendland W(q)/W(0), [wall j],
 * normal_j (walls).  Vectors have `dims` components; the rest is zero. */
aqua_status aqua_gnn_node_features(uint32_t n, int32_t dims, const float* u,
                                   const float* rho, const float* dudt,
                                   const float* drhodt, const int32_t* imove,
                                   const float* normal, const float* scales,
                                   uint16_t* out, uint32_t ld, uint32_t col,
                                   void* stream);
aqua_status aqua_gnn_edge_features(uint32_t n_edges, int32_t dims,
                                   const uint32_t* receivers,
                                   const uint32_t* senders, const float* r,
                                   const float* u, const float* rho,
                                   const int32_t* imove, const float* normal,
                                   const float* scales, uint16_t* out,
                                   void* stream);
/* The same edge features from packed node records: rec (16-byte aligned,
 * AQUA_GNN_RECORD_FLOATS(dims) floats per node) is written by
 * aqua_gnn_node_records from the node-ordered r, u, rho, imove, normal;
 * the features are bit-identical to aqua_gnn_edge_features'.  out is
 * 16-byte aligned (32-byte rows, stored as two 16-byte halves). */
#define AQUA_GNN_RECORD_FLOATS(dims) ((dims) == 3 ? 12 : 8)
aqua_status aqua_gnn_node_records(uint32_t n, int32_t dims, const float* r,
                                  const float* u, const float* rho,
                                  const int32_t* imove, const float* normal,
                                  float* rec, void* stream);
aqua_status aqua_gnn_edge_features_rec(uint32_t n_edges, int32_t dims,
                                       const uint32_t* receivers,
                                       const uint32_t* senders,
                                       const float* rec, const float* scales,
                                       uint16_t* out, void* stream);

/* ---- dense layers (tensor cores, bf16 x bf16 -> f32) ------------------- */

/* Z = X W^T + b (f32, optional), Y = act(Z) (bf16, optional).
 * X: M x K (ldx), W: N x K, b: N (optional).  K % 16 == 0, K <= 160,
 * N in {16, 64}. */
aqua_status aqua_gnn_linear_fwd(uint32_t M, uint32_t K, uint32_t N,
                                const uint16_t* X, uint32_t ldx,
                                const uint16_t* W, const float* b, float* Z,
                                uint32_t ldz, uint16_t* Y, uint32_t ldy,
                                int32_t act, void* stream);
/* The same forward on the 5th-generation tensor cores (tcgen05.mma with a
 * tensor-memory accumulator, 128-row tiles), for N = 64: all pointers
 * 16-byte aligned, ldz % 4 == 0.  Z is the FP32 accumulator plus bias; Y
 * is Z rounded to bf16 and, for SiLU, activated in packed bf16 arithmetic
 * (within a few bf16 roundings of aqua_gnn_linear_fwd's FP32 SiLU).  A
 * time-out of its bounded waits sets *err (device int, set to 0 by the
 * caller) instead of hanging. */
aqua_status aqua_gnn_linear_fwd_tc(uint32_t M, uint32_t K, uint32_t N,
                                   const uint16_t* X, uint32_t ldx,
                                   const uint16_t* W, const float* b, float* Z,
                                   uint32_t ldz, uint16_t* Y, uint32_t ldy,
                                   int32_t act, int32_t* err, void* stream);
/* A whole three-layer edge MLP on the tensor cores, activations on chip:
 * Y = L3(act3)(L2(act2)(L1(act1)(X))), 64-wide layers (W1: 64 x K1, W2, W3:
 * 64 x 64, bf16; biases f32), Y: E x 64 bf16 at ldy.  The layer-1 input is
 * the rows of X (ldx; K1 = AQUA_GNN_FEATURES, or 80 for the first node
 * MLP) or, with X = NULL, the concatenation [H[recv[e]], H[send[e]], Ef[e]]
 * (K1 = 144) that
 * aqua_gnn_gather_pair builds -- gathered on chip instead.  Bit-identical to
 * three aqua_gnn_linear_fwd_tc calls with the intermediate activations
 * rounded to bf16.  A time-out of the bounded waits sets *err. */
aqua_status aqua_gnn_edge_mlp_tc(uint32_t E, uint32_t K1, const uint16_t* X,
                                 uint32_t ldx, const uint32_t* recv,
                                 const uint32_t* send, const uint16_t* H,
                                 uint32_t ldh, const uint16_t* Ef,
                                 const uint16_t* W1, const float* b1,
                                 const uint16_t* W2, const float* b2,
                                 const uint16_t* W3, const float* b3,
                                 int32_t act1, int32_t act2, int32_t act3,
                                 uint16_t* Y, uint32_t ldy, int32_t* err,
                                 void* stream);
/* The same fused edge MLP followed by aqua_gnn_segment_sum, with the edge
 * outputs kept on chip: out[s] (64 bf16 at column col of rows ld apart) =
 * scale * sum of the layer-3 rows of node s's edges (receiver-major,
 * offsets[0..n_nodes]; recv is required in both input forms).  Each receiver
 * is summed in edge order by one CTA, so the result is bit-identical to
 * aqua_gnn_edge_mlp_tc + aqua_gnn_segment_sum, without the E x 64 bf16
 * intermediate.  E < 2^31; a time-out of the bounded waits sets *err. */
aqua_status aqua_gnn_edge_mlp_sum_tc(uint32_t n_nodes, uint32_t E, uint32_t K1,
                                     const uint16_t* X, uint32_t ldx,
                                     const uint32_t* offsets,
                                     const uint32_t* recv, const uint32_t* send,
                                     const uint16_t* H, uint32_t ldh,
                                     const uint16_t* Ef, const uint16_t* W1,
                                     const float* b1, const uint16_t* W2,
                                     const float* b2, const uint16_t* W3,
                                     const float* b3, int32_t act1,
                                     int32_t act2, int32_t act3, float scale,
                                     uint16_t* out, uint32_t ld, uint32_t col,
                                     int32_t* err, void* stream);
/* dX = dY W (M x K, bf16 at ldx) where dY: M x N bf16 (ldy), Wt: K x N.
 * With Zprev (M x K f32, ldzp) and act_prev = AQUA_ACT_SILU the result is
 * multiplied by silu'(Zprev) (the gradient of the previous layer's
 * pre-activation).  N % 16 == 0, N <= 64, K % 16 == 0, K <= 160. */
aqua_status aqua_gnn_linear_dgrad(uint32_t M, uint32_t N, uint32_t K,
                                  const uint16_t* dY, uint32_t ldy,
                                  const uint16_t* Wt, const float* Zprev,
                                  uint32_t ldzp, int32_t act_prev,
                                  uint16_t* dX, uint32_t ldx, void* stream);
/* dW += dY^T X (N x K f32), db += column sums of dY (optional).
 * dY: M x N bf16 (ldy), X: M x K bf16 (ldx); N in {16, 64}. */
aqua_status aqua_gnn_linear_wgrad(uint32_t M, uint32_t N, uint32_t K,
                                  const uint16_t* dY, uint32_t ldy,
                                  const uint16_t* X, uint32_t ldx, float* dW,
                                  float* db, void* stream);

/* aqua_gnn_linear_dgrad on the 5th-generation tensor cores (tcgen05.mma,
 * BF16 x BF16 -> FP32 in tensor memory): the same product and SiLU'
 * epilogue; N in {16, 64}, K % 16 == 0, K <= 160; rows 16-byte aligned.
 * A time-out of the bounded waits sets *err.  No counterpart in the
 * reference. */
aqua_status aqua_gnn_linear_dgrad_tc(uint32_t M, uint32_t N, uint32_t K,
                                     const uint16_t* dY, uint32_t ldy,
                                     const uint16_t* Wt, const float* Zprev,
                                     uint32_t ldzp, int32_t act_prev,
                                     uint16_t* dX, uint32_t ldx, int32_t* err,
                                     void* stream);
/* aqua_gnn_linear_wgrad on the tensor cores: dW += dY^T X (N x K f32) and
 * db += column sums of dY (optional), the reduction over the M rows in
 * chunks of 128 accumulated in tensor memory, then added with atomics;
 * N in {16, 64}, K % 16 == 0, K <= 160.  A time-out sets *err. */
aqua_status aqua_gnn_linear_wgrad_tc(uint32_t M, uint32_t N, uint32_t K,
                                     const uint16_t* dY, uint32_t ldy,
                                     const uint16_t* X, uint32_t ldx,
                                     float* dW, float* db, int32_t* err,
                                     void* stream);

/* ---- graph aggregation ------------------------------------------------- */

/* out[s] = scale * sum of Y rows of node s's edges (64 wide, bf16 out at
 * column `col` of rows ld apart). */
aqua_status aqua_gnn_segment_sum(uint32_t n_nodes, const uint32_t* offsets,
                                 const uint16_t* Y, uint32_t ldy, float scale,
                                 uint16_t* out, uint32_t ld, uint32_t col,
                                 void* stream);
/* dY[e] = scale * dAgg[receiver(e)] (64 wide bf16; dAgg at column col of
 * rows ld apart) -- the gradient of aqua_gnn_segment_sum. */
aqua_status aqua_gnn_segment_bcast(uint32_t n_edges, const uint32_t* receivers,
                                   const uint16_t* dAgg, uint32_t ld,
                                   uint32_t col, float scale, uint16_t* dY,
                                   uint32_t ldy, void* stream);
/* Edge rows of the second round: [H[receiver], H[sender], E] (144 wide). */
aqua_status aqua_gnn_gather_pair(uint32_t n_edges, const uint32_t* receivers,
                                 const uint32_t* senders, const uint16_t* H,
                                 uint32_t ldh, const uint16_t* E,
                                 uint16_t* out, void* stream);
/* Gradient of aqua_gnn_gather_pair into the node latents:
 * dH[s] += sum over s's edges of dX[e][0:64] and, for every edge e,
 * dH[sender(e)] += dX[e][64:128]  (dH f32, 64 wide). */
aqua_status aqua_gnn_scatter_pair(uint32_t n_nodes, uint32_t n_edges,
                                  const uint32_t* offsets,
                                  const uint32_t* senders, const uint16_t* dX,
                                  float* dH, void* stream);
/* dst (bf16, at column col of rows ld apart) = src (f32 n x 64) + extra
 * (bf16 n x 64 at column ecol of rows eld apart, optional) */
aqua_status aqua_gnn_add_to_bf16(uint32_t n, const float* src,
                                 const uint16_t* extra, uint32_t eld,
                                 uint32_t ecol, uint16_t* dst, uint32_t ld,
                                 uint32_t col, void* stream);

/* ---- loss and optimiser ------------------------------------------------ */

/* Masked mean squared error of the first `t` output columns (out f32 n x 16)
 * against target (f32 n x t) over nodes with mask != 0: loss (f32, atomic
 * add) = sum / count; dOut (bf16 n x 16) = 2 (out - target) / count on
 * masked rows, 0 elsewhere. */
aqua_status aqua_gnn_mse(uint32_t n, uint32_t t, const float* out,
                         const float* target, const int32_t* mask,
                         float count, float* loss, uint16_t* dOut,
                         void* stream);
/* Adam step on f32 master weights w (gradient g, moments m, v; step >= 1);
 * also writes the bf16 copy. */
aqua_status aqua_gnn_adam(uint32_t n, float* w, const float* g, float* m,
                          float* v, float lr, float beta1, float beta2,
                          float eps, uint32_t step, uint16_t* w_bf16,
                          void* stream);
/* f32 -> bf16 (round to nearest even), and the K x N transpose of an N x K
 * bf16 matrix */
aqua_status aqua_gnn_to_bf16(uint32_t n, const float* src, uint16_t* dst,
                             void* stream);
aqua_status aqua_gnn_transpose(uint32_t N, uint32_t K, const uint16_t* W,
                               uint16_t* Wt, void* stream);

/* ---- proposal ---------------------------------------------------------- */

/* For fluid particles (imove == 1): u' = u + T dudt + su * out[0:dims],
 * rho' = rho + T drhodt + srho * out[dims], r' = r + T (u + u') / 2,
 * T = k * dt of the particle's case (dt_case[cid]); node-ordered `out`
 * (node s = particle perm[s]).  Walls and probes keep r, u, rho here. */
aqua_status aqua_gnn_apply(uint32_t n_nodes, int32_t dims,
                           const uint32_t* perm, const float* out,
                           const uint32_t* cid, const float* dt_case,
                           uint32_t k, float su, float srho, float* r,
                           float* u, float* rho, const float* dudt,
                           const float* drhodt, const int32_t* imove,
                           void* stream);

/* Training targets of fluid nodes (mask = 1; other nodes mask = 0,
 * target 0): target[s] = ((u1 - u0 - T dudt0) / su, (rho1 - rho0 -
 * T drhodt0) / srho), T = k * dt_case[cid], arrays per particle, node s =
 * particle perm[s]; target is n_nodes x (dims + 1). */
aqua_status aqua_gnn_targets(uint32_t n_nodes, int32_t dims,
                             const uint32_t* perm, const float* u0,
                             const float* rho0, const float* dudt0,
                             const float* drhodt0, const float* u1,
                             const float* rho1, const uint32_t* cid,
                             const float* dt_case, uint32_t k, float su,
                             float srho, const int32_t* imove, float* target,
                             int32_t* mask, void* stream);
/* Prescribed roll of the walls and probes (imove != 1) of set roll[c].iset
 * of case c from angle psi0[c] to psi1[c] about center (z axis): r, normal
 * and tangent rotated by psi1 - psi0, velocity omega1[c] x (r - center).
 * Per-case device arrays: enabled (i32), iset (u32), psi0, psi1, omega1
 * (f32), center (f32 x 4). */
aqua_status aqua_gnn_roll(uint32_t n, int32_t dims, const uint32_t* cid,
                          const uint32_t* iset, const int32_t* imove,
                          const int32_t* enabled, const uint32_t* roll_iset,
                          const float* psi0, const float* psi1,
                          const float* omega1, const float* center4,
                          float* r, float* normal, float* tangent, float* u,
                          void* stream);
/* Probe pressure of each case c (particles [offsets[c], offsets[c+1]) in
 * any order): at the case's first probe (imove == 0), the Shepard-
 * normalised interpolation of the fluid pressure p_j = p0 + cs^2 (rho_j -
 * refd) (the reference's cfd/Sensors.cl and SensorsRenormalization.cl with
 * the linear EOS): sum p_j W_ij CONW m_j / rho_j over fluid j within
 * SUPPORT * H, divided by the Shepard sum (1 when below 1e-6).  consts
 * (host memory) = H, CONW, SUPPORT, cs, p0, refd.  out[c] = 0 for a case
 * without probe. */
aqua_status aqua_gnn_probe_pressure(uint32_t n_cases, int32_t dims,
                                    const uint32_t* offsets, const float* r,
                                    const float* rho, const float* m,
                                    const int32_t* imove, const float* consts,
                                    float* out, void* stream);
/* Pressure at several probes of one case: for each probe k (the particle
 * probe[k] of the arrays, at most AQUA_GNN_MAX_PROBES), the same Shepard-
 * normalised interpolation as aqua_gnn_probe_pressure over the fluid
 * particles of [0, n).  The sums are reduced in a fixed order (a fixed grid
 * of AQUA_GNN_PROBE_BLOCKS blocks, then the blocks in order): the result is
 * deterministic.  scratch: AQUA_GNN_PROBE_SCRATCH floats of device memory;
 * consts (host memory) as for aqua_gnn_probe_pressure. */
#define AQUA_GNN_MAX_PROBES 8
#define AQUA_GNN_PROBE_BLOCKS 256
#define AQUA_GNN_PROBE_SCRATCH (2 * AQUA_GNN_MAX_PROBES * AQUA_GNN_PROBE_BLOCKS)
aqua_status aqua_gnn_probes_pressure(uint32_t n, int32_t dims, const float* r,
                                     const float* rho, const float* m,
                                     const int32_t* imove, uint32_t n_probes,
                                     const uint32_t* probe, const float* consts,
                                     float* scratch, float* out, void* stream);
/* *out (device float) = max of |a_i - b_i| * scale over a random subsample
 * of the fluid particles (imove == 1) of [0, n): particle i is in it when a
 * 32-bit hash of (i, seed) falls below fraction * 2^32, so about `fraction`
 * of them, drawn anew for each seed; a non-finite difference counts as
 * infinite.  Deterministic for a given seed. */
aqua_status aqua_gnn_sample_max_diff(uint32_t n, const float* a,
                                     const float* b, const int32_t* imove,
                                     uint32_t seed, float fraction, float scale,
                                     float* out, void* stream);
/* The judge of a proposal on a rate sample (aqua_set_rate_sample with
 * `fraction` and `seed`): a solver stepped once from the start state s0 and
 * once from the proposed state s1 (k steps of dt later), each with the
 * sample on, holds the plain rates drho/dt of the sampled cells at both
 * ends.  For every particle, rho_judged[id] = rho0 + kdt/2 (drhodt0 +
 * drhodt1): the density the plain continuity equation gives over the k
 * steps (trapezoidal rule).  *out = max |rho1 - rho_judged| * scale over the
 * fluid particles in sampled cells at both ends.  Inputs: id1, icell1 (cell
 * keys), imove1, drhodt1 in the sorted order of the s1 step; icell0,
 * drhodt0 of the s0 step and rho0, rho1 (s0, s1) by particle id; rho_judged
 * by particle id. */
aqua_status aqua_gnn_judge_density(uint32_t n, const uint32_t* id1,
                                   const uint32_t* icell1, const int32_t* imove1,
                                   const float* drhodt1, const uint32_t* icell0,
                                   const float* drhodt0, const float* rho0,
                                   const float* rho1, float kdt, float scale,
                                   float fraction, uint32_t seed,
                                   float* rho_judged, float* out, void* stream);
/* out[c] = max over fluid particles i of case c of |a_i - b_i| * scale */
aqua_status aqua_gnn_case_max_diff(uint32_t n_cases, const uint32_t* offsets,
                                   const float* a, const float* b,
                                   const int32_t* imove, float scale,
                                   float* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif
