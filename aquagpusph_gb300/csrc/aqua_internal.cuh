// Internal declarations of the aqua_gb300 CUDA library (sm_103a).
//
// Floating point contract: the library is compiled with -fmad=false and the
// default IEEE division / square root, so each multiply, add, divide and
// square root is one correctly rounded binary32 operation in source order,
// exactly as the reference's kernels write them (and as the CPU oracle
// restates them).  Summation order per particle follows the reference's
// neighbour-visiting order (types/3D.h:197-219: 27 cells, x offset
// outermost; particles of a cell in sorted order).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "aqua_gb300.h"

namespace aqua {

constexpr int kMaxSets = 16;

// test-only switch of aqua_debug_fake_timeouts() (api.cu): bounded waits
// that completed report a time-out
extern int g_debug_fake_timeout;

// Error word bits written by kernels (read back by aqua_check)
enum : uint32_t
{
    kErrCapacity = 1u << 0,
    kErrDt = 1u << 1,
    kErrNonFinite = 1u << 2,
    kErrTimeout = 1u << 3,   // a bounded wait in a kernel ran out
};

// Case constants as the kernels see them (__constant__ copy per launch set)
struct Consts
{
    int dims;
    uint32_t n_sets;
    float h, support, H, CONW, CONF, SUPPORT, DIMS;
    float cs, p0;
    float g[4];
    float courant, dt_Ma, dt_min, dt_fixed;
    float domain_min[4], domain_max[4];
    float dr_factor, min_bound_dist, relax_midpoint;
    uint32_t iter_midpoint_max;
    float refd[kMaxSets], visc_dyn[kMaxSets], delta[kMaxSets];
    int boundary;       // AQUA_BOUNDARY_BIE or AQUA_BOUNDARY_BI
    int scheme;         // AQUA_SCHEME_MIDPOINT or AQUA_SCHEME_IMPROVED_EULER
    // derived
    float cell_length;  // support * h (LinkList.cpp:156)
    float idist;        // 1 / (support * h) (LinkList.cl.in:73)
    float q2_reject;    // |r_ij|^2 >= q2_reject  =>  |r_ij| / H >= SUPPORT
    // folded factors of the fast build's pair sums
    float inv_H;        // 1 / H
    float w_conw;       // W factor of the Wendland kernel * CONW
    float f_conf;       // F factor * CONF
    float f_over_w;     // f_conf / w_conw (clustered sweep)
    // test-only: a bounded wait that completed is reported as timed out
    // (AQUA_ERR_TIMEOUT), so the error path runs with nothing in flight
    uint32_t debug_fake_timeout;
    // rate sample (aqua_set_rate_sample): the clustered sweep runs only the
    // cells whose key hashes below sample_thr, and every cell around a probe
    uint32_t sample_on;
    uint32_t sample_thr;
    uint32_t sample_seed;
};

// 32-bit hash of a cell key for the rate sample (host and device)
__host__ __device__ inline uint32_t
sample_hash(uint32_t key, uint32_t seed)
{
    uint32_t h = key * 0x9E3779B1u ^ (seed * 0x85EBCA77u + 0x165667B1u);
    h ^= h >> 16;
    h *= 0x85EBCA6Bu;
    h ^= h >> 13;
    h *= 0xC2B2AE35u;
    h ^= h >> 16;
    return h;
}

// Device-side scalars of one case of the resident state (a batch holds
// n_cases independent cases, each with its own link-list and time step)
struct CaseScalars
{
    float r_min[4];
    float r_max[4];
    uint32_t n_cells[4];
    uint32_t cell_base;  // first global cell key of the case
    float t;
    float dt;            // time step of the step being run
    uint32_t dt_next;    // bits of the running minimum of dt_var (atomicMin)
    uint32_t iter;
    float psi;           // roll angle of the moving boundary (rad)
    float psi_in;        // roll angle of the previous step
    float omega;         // roll rate (rad/s)
    // cos / sin of psi and psi_in, evaluated in double and rounded
    float cos_psi, sin_psi, cos_psi_in, sin_psi_in;
};

// Prescribed roll of a case's boundary elements and probes about `center`
// (z axis): psi(t) = amplitude * sin(angular_freq * t)
struct CaseMotion
{
    int32_t enabled;
    uint32_t iset;       // the particle set that moves (non-fluid particles)
    float amplitude;
    float angular_freq;
    float center[4];
};

// Device-side scalars shared by all cases
struct DevScalars
{
    uint32_t err;         // error bits
    uint32_t n_chunks;    // cell-aligned sweep chunks of this step
    uint32_t chunk_next;  // next chunk to hand out (work counter)
    uint32_t total_cells; // cells of all cases
    uint32_t pad[4];
};

// One set of the per-particle Variables (reference layout)
struct VarSet
{
    uint32_t* cid;   // case of each particle (batched runs)
    uint32_t* id;
    uint32_t* iset;
    int32_t* imove;
    float* r;
    float* normal;
    float* tangent;
    float* binormal;
    float* u;
    float* dudt;
    float* rho;
    float* drhodt;
    float* m;
    float* p;
};

// Per-step scratch of the link-list and the sweep
struct StepBufs
{
    // link-list
    uint32_t* keys[2];     // radix ping-pong keys
    uint32_t* vals[2];     // radix ping-pong values (original index)
    uint32_t* sort_scratch; // digit histograms, tile counters, look-back
                            // status (sort_scratch_words)
    uint2* cells;          // (start, end) per cell; (N, N) if empty
    uint2* chunks;         // (first, count) sweep chunks (<= N)
    uint2* wall_range;     // first and one past the last sorted index of the
                           // cell's boundary elements; (~0, 0) if none
    uint32_t* id_sorted;   // old -> new
    // sorted start-of-step Variables (the reference's *_in after the
    // midpoint backups)
    float* r_in;
    float* u_in;
    float* dudt_in;
    float* rho_in;
    float* drhodt_in;
    // packed neighbour data (sorted): position + imove, half-step velocity
    // + density, pressure + mass
    float4* posq;
    float4* velq;
    float2* pmq;
    // optional intermediates (written when extras are on)
    float* grad_p;
    float* lap_u;
    float* div_u;
    float* lap_p;
    float* grad_w_bi;
    float* div_u_bi;
    float* shepard;
    // clustered sweep (fast build, 3-D): per sorted particle two 16-byte
    // neighbour records, rec0 = (x, y, z, w) with w = CONW * W-factor * m/rho
    // (fluid), -m
    // (boundary element, its area) or 0 (no neighbour sums), rec1 = (u, p)
    // (fluid) or (normal, u.normal) (boundary element); the cells holding
    // particles as (key, first sorted index) in `work`, their cluster
    // ranges in `wcl` (first, end, case, clusters; the cell's clusters
    // start at index `first` of `clu`), the (first sorted index, count) of
    // the 9 rows of 3 cells around each in `crow`; clusters of <= 8
    // particles of one cell octant as (first position in cperm, count);
    // cperm = sorted indices in cluster order
    float4* rec0;
    float4* rec1;
    uint8_t* cell_mark;    // rate sample: cells around a probe (ncap)
    uint2* work;
    uint4* wcl;
    uint2* crow;           // 9 per listed cell (ncap cells at most)
    uint2* clu;
    uint32_t* cperm;
};

}  // namespace aqua
