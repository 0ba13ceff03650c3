/*
 * aqua_gb300 -- GB300 (sm_103a) CUDA implementation of AQUAgpusph's per-step
 * WCSPH particle pipeline, behind a plain C ABI.
 *
 * The reference runs the step as a list of OpenCL tools configured by XML
 * presets (basic.xml:132-171 plus the midpoint, domain, cfd, deltaSPH, BIe
 * and variableTimeStep presets).  This library replaces the tools of that
 * path:
 *
 *   reference tool(s)                                   entry point here
 *   --------------------------------------------------  --------------------
 *   link-list (LinkList.cpp:326-494: Reduction min/max,  aqua_linklist()
 *     nCells, iCell, RadixSort, iHoc, linkList)
 *   radix-sort (RadixSort.cpp:130-304)                   aqua_radix_sort()
 *   predictor, Domain, link-list, Backup*, sort stage1/2, aqua_step()
 *     EOS, Binormal, reinit sets, midpoint loop (advance,
 *     eos, cfd Shepard/interactions/sensors/lap p, BIe
 *     interactions/rates, cfd rates, delta-SPH, elastic
 *     bounce, relax), corrector, BIe pst, time step,
 *     minimum time step reduction, t += dt
 *
 * Conventions
 *   - extern "C", POD arguments only; no exception crosses the ABI.
 *   - every function returns an aqua_status (0 = success, negative = error).
 *   - device pointers unless a name says "host".
 *   - `vec` arrays hold float4 per particle in 3-D and float2 in 2-D (the
 *     reference's vec type); index arrays are uint32 (the reference's usize
 *     on 32-bit-address devices, CalcServer.cpp:260-264).
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy stream).
 *   - A context lives on the device that was current at aqua_create().
 */
#ifndef AQUA_GB300_H
#define AQUA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum
{
    AQUA_OK = 0,
    AQUA_ERR_INVALID = -1,     /* bad argument */
    AQUA_ERR_CAPACITY = -2,    /* n_cells exceeds the ihoc capacity */
    AQUA_ERR_DT = -3,          /* time step not > 0 (variableTimeStep.xml:16) */
    AQUA_ERR_CUDA = -4,        /* a CUDA runtime call failed */
    AQUA_ERR_NO_MEMORY = -5,   /* device allocation failed */
    AQUA_ERR_NONFINITE = -6,   /* non-finite position reached the link-list */
    AQUA_ERR_IO = -7,          /* a file could not be opened or read */
    AQUA_ERR_FORMAT = -8,      /* a particles file line is malformed */
    AQUA_ERR_TIMEOUT = -9      /* a bounded wait inside a kernel ran out */
} aqua_status;

/* Scalar Variables and Definitions of one case.  The Definitions are the
 * compiled values: CalcServer.cpp:247-257 bakes evaluated expressions in as
 * "%#G" literals, so H, CONW, CONF and DIMS carry six significant digits. */
typedef struct
{
    int32_t dims;              /* 2 or 3 */
    uint32_t n_sets;           /* length of refd / visc_dyn / delta */
    float h;                   /* Variable h */
    float support;             /* Variable support (kernel support / h) */
    float H;                   /* Definition H */
    float CONW;                /* Definition CONW = 1/h^dims */
    float CONF;                /* Definition CONF = 1/h^(dims+2) */
    float SUPPORT;             /* Definition SUPPORT */
    float DIMS;                /* Definition DIMS */
    float cs;                  /* Variable cs (speed of sound) */
    float p0;                  /* Variable p0 (background pressure) */
    float g[4];                /* Variable g (gravity) */
    float courant;             /* Variable courant */
    float dt_Ma;               /* Variable dt_Ma */
    float dt_min;              /* Variable dt_min */
    float dt_fixed;            /* "fixed time step" = courant*h/cs */
    float domain_min[4];       /* Variable domain_min */
    float domain_max[4];       /* Variable domain_max */
    float dr_factor;           /* Definition __DR_FACTOR__ */
    float min_bound_dist;      /* Definition __MIN_BOUND_DIST__ */
    float relax_midpoint;      /* Variable relax_midpoint */
    uint32_t iter_midpoint_max; /* Variable iter_midpoint_max */
    const float* refd;         /* host, n_sets: per-set reference density */
    const float* visc_dyn;     /* host, n_sets: dynamic viscosity */
    const float* delta;        /* host, n_sets: delta-SPH factor */
    int32_t boundary;          /* wall formulation: AQUA_BOUNDARY_BIE (the
                                  canonical cfd/BIe.xml) or AQUA_BOUNDARY_BI
                                  (cfd/BI.xml: analytic Shepard factor,
                                  free-slip boundary integrals) */
    int32_t scheme;            /* time scheme: AQUA_SCHEME_MIDPOINT (the
                                  canonical basic/time_scheme/midpoint.xml,
                                  iter_midpoint_max = 1) or
                                  AQUA_SCHEME_IMPROVED_EULER
                                  (basic/time_scheme/improved_euler.xml;
                                  BI walls only, as in every reference example
                                  that uses it -- with BIe walls the elastic
                                  bounce would read the predictor's unsorted
                                  r_in/u_in by sorted index) */
} aqua_params;

#define AQUA_BOUNDARY_BIE 0
#define AQUA_BOUNDARY_BI 1
#define AQUA_SCHEME_MIDPOINT 0
#define AQUA_SCHEME_IMPROVED_EULER 1

/* The particle Variables of one case (all length N; pointers may be host or
 * device memory as each function states).  Fields a call does not use may
 * be NULL. */
typedef struct
{
    uint32_t* id;
    uint32_t* iset;
    int32_t* imove;
    float* r;          /* vec */
    float* normal;     /* vec */
    float* tangent;    /* vec */
    float* binormal;   /* vec */
    float* u;          /* vec */
    float* dudt;       /* vec */
    float* rho;
    float* drhodt;
    float* m;
    float* p;
    float* shepard;
} aqua_vars;

/* Variables a step leaves behind besides the state (the reference keeps
 * them as Variables too): backups, link-list tables and the step's
 * intermediate operators.  Used by aqua_get_extra(). */
typedef struct
{
    float* r_in;       /* vec, sorted start-of-step positions */
    float* u_in;       /* vec */
    float* dudt_in;    /* vec */
    float* rho_in;
    float* drhodt_in;
    uint32_t* icell;   /* sorted cell of each particle */
    uint32_t* id_sorted;   /* old index -> sorted index */
    uint32_t* id_unsorted; /* sorted index -> old index */
    uint32_t* ihoc;    /* head of chain of each cell, N if empty (n_cells.w) */
    float* grad_p;     /* vec, after the BIe rates */
    float* lap_u;      /* vec */
    float* div_u;      /* after the BIe rates */
    float* lap_p;
    float* grad_w_bi;  /* vec */
    float* div_u_bi;
} aqua_extra;

/* Scalars of the resident state */
typedef struct
{
    float t;
    float dt;
    uint32_t iter;
    uint32_t n_cells[4];
    float r_min[4];
    float r_max[4];
} aqua_scalars;

/* One case of a batch: its scalars and an optional prescribed roll of its
 * boundary elements and probes (particles of set `roll_iset` that are not
 * fluid) about the z axis through `roll_center`:
 * psi(t) = roll_amplitude * sin(roll_angular_freq * t).  The motion is
 * applied at the end of every step, after the time step, as the reference's
 * motion preset does (cfd/motion.xml:59-71). */
typedef struct
{
    float t;
    float dt;
    uint32_t iter;
    int32_t roll_enabled;
    uint32_t roll_iset;
    float roll_amplitude;     /* rad */
    float roll_angular_freq;  /* rad/s */
    float roll_center[4];
} aqua_case;

typedef struct aqua_ctx aqua_ctx;

/* Library version string */
const char* aqua_version(void);

/* Device memory for bindings that have no CUDA runtime of their own (ctypes,
 * JNI, a host tool): allocate, free, and copy with a wait.  kind:
 * AQUA_COPY_H2D, AQUA_COPY_D2H or AQUA_COPY_D2D. */
#define AQUA_COPY_H2D 0
#define AQUA_COPY_D2H 1
#define AQUA_COPY_D2D 2
aqua_status aqua_malloc(void** ptr, size_t bytes);
aqua_status aqua_free(void* ptr);
aqua_status aqua_memcpy(void* dst, const void* src, size_t bytes, int kind);

/* Creates a context for cases of up to `capacity` particles on the current
 * device.  `ihoc_capacity` bounds n_cells.w (0 = derive it from the domain
 * box in `params`).  Allocates all device memory the step needs; no later
 * call allocates.  (CalcServer::setup, CalcServer.cpp:1435-1534, and
 * LinkList::setup / allocate, LinkList.cpp:137-183, 234-271.) */
aqua_status aqua_create(const aqua_params* params, uint32_t capacity,
                        uint32_t ihoc_capacity, aqua_ctx** out);
aqua_status aqua_destroy(aqua_ctx* ctx);

/* Replaces the case parameters (same dims and ihoc capacity). */
aqua_status aqua_set_params(aqua_ctx* ctx, const aqua_params* params);

/* With `on` = 1 every step also stores the intermediate operators (grad_p,
 * lap_u, div_u, lap_p, grad_w_bi, div_u_bi) the reference keeps as
 * Variables, for aqua_get_extra(); off by default (the fused step does not
 * need them). */
aqua_status aqua_set_extras(aqua_ctx* ctx, int on);

/* Arithmetic of the step kernels.  AQUA_PRECISION_EXACT (the default):
 * every operation of the reference's kernels as one correctly rounded IEEE
 * binary32 operation in the reference's order, no FMA contraction -- the
 * results equal the reference kernels' bit for bit (positions up to the
 * last bit of powf in the BIe PST).  AQUA_PRECISION_FAST: the same kernels
 * compiled with FMA contraction and approximate division / square root;
 * per-step rates stay within 1e-5 relative of the exact ones. */
#define AQUA_PRECISION_EXACT 0
#define AQUA_PRECISION_FAST 1
aqua_status aqua_set_precision(aqua_ctx* ctx, int mode);

/* Launch shape of the sweep: `sweep_variant` selects threads per block,
 * queued neighbours per thread, the queue entry and how candidate groups
 * reach shared memory (0: 128 x 128 16-bit loads, 1: 64 x 128 16-bit loads,
 * 2: 64 x 64 32-bit loads, 3: 64 x 128 16-bit bulk copies, 4: 64 x 64
 * 32-bit bulk copies), or the direct sweep that sums each candidate group
 * as it is loaded, without a queue (5: 64 threads, 6: 128 threads; 7: 64
 * and 8: 128 threads with the next group prefetched by asynchronous
 * copies; 9: 64 and 10: 128 threads of those compiled for 28 resident warps
 * per SM, 11 and 12 for 32, 13 and 14 for 36);
 * `blocks_per_sm` the persistent grid (blocks per SM, <= 32).
 * Any choice gives the same results; aquagpusph_gb300.autotune picks the
 * fastest for a case by timing them. */
aqua_status aqua_set_tuning(aqua_ctx* ctx, uint32_t sweep_variant,
                            uint32_t blocks_per_sm);

/* Uploads the particle Variables of an N-particle case into the resident
 * state (the ParticlesSet loaders, FileManager.cpp:136-139).  `on_host` = 1
 * for host pointers, 0 for device pointers.  The call does not synchronise:
 * from pinned host memory the copies run asynchronously on `stream`, so the
 * buffers must stay unchanged until the stream has executed them (pageable
 * buffers are staged before the call returns).  Required fields: id, iset,
 * imove, r, normal, tangent, u, dudt, rho, drhodt, m, p.  binormal may be
 * NULL.  Also sets t, dt, iter. */
aqua_status aqua_set_state(aqua_ctx* ctx, uint32_t N, const aqua_vars* src,
                           int on_host, float t, float dt, uint32_t iter,
                           void* stream);

/* Splits the resident particles (uploaded by aqua_set_state) into n_cases
 * independent cases: case k holds particles [offsets[k], offsets[k+1]).
 * Every case gets its own bounding box, cell grid, sort keys, time step and
 * time; one aqua_step() advances all of them (one launch per kernel for the
 * whole batch).  Host arrays; at most 4096 cases. */
aqua_status aqua_set_cases(aqua_ctx* ctx, uint32_t n_cases,
                           const uint32_t* offsets, const aqua_case* cases,
                           void* stream);
/* Scalars of cases [first, first+count) (synchronises `stream`). */
aqua_status aqua_get_case_scalars(aqua_ctx* ctx, uint32_t first, uint32_t count,
                                  aqua_scalars* out, void* stream);

/* Copies the resident state out (any non-NULL field is written). */
aqua_status aqua_get_state(aqua_ctx* ctx, aqua_vars* dst, int on_host,
                           void* stream);
aqua_status aqua_get_extra(aqua_ctx* ctx, aqua_extra* dst, int on_host,
                           void* stream);
/* Synchronises `stream` and reads the scalars. */
aqua_status aqua_get_scalars(aqua_ctx* ctx, aqua_scalars* out, void* stream);

/* Advances the resident state by `nsteps` full canonical steps (the tool
 * list of CalcServer::update, CalcServer.cpp:592-623, for one step each).
 * Launch-only: no host synchronisation; dt stays on the device.  With
 * `use_graph` = 1 the step is captured once into a CUDA graph per parity
 * of the step and replayed. */
aqua_status aqua_step(aqua_ctx* ctx, uint32_t nsteps, int use_graph,
                      void* stream);

/* Synchronises `stream` and returns the first error a kernel recorded since
 * the last call (AQUA_ERR_CAPACITY, AQUA_ERR_DT, AQUA_ERR_NONFINITE,
 * AQUA_ERR_TIMEOUT), then clears it.  The step skips its remaining work
 * once an error is set. */
aqua_status aqua_check(aqua_ctx* ctx, void* stream);

/* The link-list tool on caller-owned device buffers (LinkList.cpp:326-494):
 * r_min/r_max of r_in over all N particles, n_cells = floor((max - min) /
 * (support*h)) + 6 per axis, icell of every particle, a stable sort of icell
 * (id_unsorted[s] = original index, id_sorted[orig] = s) and ihoc (N for an
 * empty cell).  Outputs: icell (N, sorted), id_sorted (N), id_unsorted (N),
 * ihoc (ihoc_capacity; n_cells.w entries written), host n_cells[4],
 * r_min[4], r_max[4].  Synchronises `stream` once (the reference's
 * LinkList also waits for its reductions, LinkList.cpp:350-356). */
aqua_status aqua_linklist(aqua_ctx* ctx, const float* r_in, uint32_t N,
                          uint32_t* icell, uint32_t* id_sorted,
                          uint32_t* id_unsorted, uint32_t* ihoc,
                          uint32_t ihoc_capacity, uint32_t* n_cells_host,
                          float* r_min_host, float* r_max_host,
                          void* stream);

/* The radix-sort tool on caller device buffers (RadixSort.cpp:130-304):
 * stable ascending sort of n keys below 2^key_bits (keys sorted in place),
 * perm[s] = original index, inv_perm[orig] = s (either may be NULL). */
aqua_status aqua_radix_sort(aqua_ctx* ctx, uint32_t* keys, uint32_t* perm,
                            uint32_t* inv_perm, uint32_t n, uint32_t key_bits,
                            void* stream);

/* With `on` = 1 each step records CUDA events at its stage boundaries (also
 * inside captured graphs); aqua_stage_times() then returns, for the last
 * step, the milliseconds of [0] link-list (bounding box, hash, sort),
 * [1] gather, [2] sweep, [3] finalize.  Profiling plays the role of the
 * reference's per-tool EventProfile (Kernel.cpp:38-116). */
aqua_status aqua_set_profiling(aqua_ctx* ctx, int on);
aqua_status aqua_stage_times(aqua_ctx* ctx, float* ms, uint32_t n);

/* Rate sample for judging a proposed state (no counterpart in the
 * reference): with 0 < fraction < 1, the steps of the fast 3-D build
 * (clustered sweep) evaluate the neighbour sums, rates and integrator only
 * for the particles of the cells whose key hashes (sample_hash of the key
 * and `seed`) below fraction * 2^32, about `fraction` of them, and of every
 * cell around a probe; the other particles keep the values the gather left
 * (positions, velocities and densities of the start of the step, the last
 * rates).  Stepping a state with dt = 0 this way evaluates the plain rates
 * of that state on the sample.  fraction >= 1 turns it off. */
aqua_status aqua_set_rate_sample(aqua_ctx* ctx, float fraction, uint32_t seed);

/* Test-only: with `on` = 1, every bounded wait of the library's kernels
 * (bulk-copy and tensor-core completions on an mbarrier) that completed is
 * then reported as timed out, so that the time-out path (error word ->
 * AQUA_ERR_TIMEOUT from aqua_check / the learned entry points, the state
 * left as it was) runs with no copy or MMA left in flight.  Process-wide;
 * read when steps are enqueued (a CUDA graph keeps the value it was
 * captured with).  No counterpart in the reference. */
aqua_status aqua_debug_fake_timeouts(int on);

/* The stable radix sort of aqua_radix_sort(), for callers that cannot
 * allocate device memory: a tool inside another runtime's pre-sized step
 * loop, code running while a stream is captured, a process held to a fixed
 * device-memory budget.  No context, no cudaMalloc, no allocating library
 * call.  It has no counterpart in the reference.  Its scratch is a
 * fixed-size array of the library, 13.11 MB (3 * 2^20 + 2^17 + 1,056
 * 32-bit words), held by every CUDA context that uses it until the context
 * ends,
 * so n is limited to AQUA_NOALLOC_SORT_MAX_KEYS; larger n returns
 * AQUA_ERR_CAPACITY.  keys are sorted in place (values below 2^key_bits),
 * perm[s] = original index and inv_perm[orig] = s (either may be NULL).
 * All calls in a context share the scratch: calls that overlap on the GPU
 * race.  The first call in each CUDA context (contexts are told apart by
 * their unique id, so a driver-API host's own context and a primary context
 * re-created after cudaDeviceReset each count as new) looks the scratch
 * address up, and it is also where the array's memory is committed, since
 * CUDA loads modules lazily: under a fixed budget that first call is the
 * one that can fail.  Make it before any stream capture; a call that would
 * need the lookup while `stream` is capturing returns AQUA_ERR_INVALID and
 * launches nothing. */
#define AQUA_NOALLOC_SORT_MAX_KEYS (1u << 20)
aqua_status aqua_radix_sort_noalloc(uint32_t* keys, uint32_t* perm,
                                    uint32_t* inv_perm, uint32_t n,
                                    uint32_t key_bits, void* stream);

/* Fields of the resident state for aqua_get_unsorted(). */
#define AQUA_FIELD_R 0        /* vec */
#define AQUA_FIELD_NORMAL 1   /* vec */
#define AQUA_FIELD_TANGENT 2  /* vec */
#define AQUA_FIELD_U 3        /* vec */
#define AQUA_FIELD_DUDT 4     /* vec */
#define AQUA_FIELD_RHO 5
#define AQUA_FIELD_DRHODT 6
#define AQUA_FIELD_M 7
#define AQUA_FIELD_P 8
#define AQUA_FIELD_SHEPARD 9
#define AQUA_FIELD_IMOVE 10   /* int32 values */
/* Report staging limit of aqua_get_unsorted() into host memory (values) */
#define AQUA_REPORT_MAX_VALUES (1u << 20)

/* The values of one field for the particles whose original index (the id
 * given at aqua_set_state) lies in [first, first + n), in original order:
 * out[(id - first) * nc + k], nc = components of the field (2 or 4 for vec,
 * else 1), 32-bit values.  The reference's particle reports read their
 * fields this way (CalcServer::getUnsortedMem, used by SetTabFile.cpp:
 * 282-287).  `on_host` = 1: out is host memory, n * nc <=
 * AQUA_REPORT_MAX_VALUES (else AQUA_ERR_CAPACITY), and the call synchronises
 * `stream`; 0: out is device memory and the call only enqueues. */
aqua_status aqua_get_unsorted(aqua_ctx* ctx, int field, uint32_t first,
                              uint32_t n, void* out, int on_host,
                              void* stream);

/* Free-surface elevation sensors, as the wave-height sensors of the 3-D
 * dam-break example (examples/3D/spheric_testcase2_dambreak/src/templates/
 * h_sensor.cl:37-61 and the max reductions of Sensors.xml:43-62): for
 * sensor k at horizontal position sensors[2k], sensors[2k+1] (x, y; y unused
 * in 2-D), out[k] = max over particles of h_i, where h_i = r_i[up] + dr/2
 * for fluid particles (imove > 0) with |x_i - x_k| <= 2 dr (and |y_i - y_k|
 * <= 2 dr in 3-D) and 0 for every other particle; up = y in 2-D, z in 3-D.
 * case_index >= 0 restricts the maximum to that case of a batch (-1: all
 * particles).  At most 64 sensors; out is host memory; synchronises. */
aqua_status aqua_free_surface(aqua_ctx* ctx, const float* sensors,
                              uint32_t n_sensors, float dr, int32_t case_index,
                              float* out, void* stream);

/* Column types of aqua_read_fastascii() */
#define AQUA_COLUMN_FLOAT 0   /* float and vec fields */
#define AQUA_COLUMN_INT 1     /* int fields (imove) */
#define AQUA_COLUMN_UINT 2    /* unsigned int fields */

/* Reads a FastASCII particles file (InputOutput/FastASCII.cpp and the line
 * rules of InputOutput/ASCII.cpp:65-240, 374-403): comments from '#', the
 * separators " ;()[]{}\t," (runs count once), one particle per non-empty
 * line with exactly n_cols numbers of the given column types.  Host only, no
 * GPU.  out = NULL: *n_rows = number of particle lines (no parsing).
 * Otherwise the numbers go to out as 32-bit words, row-major
 * (n_rows x n_cols, at most max_rows rows, else AQUA_ERR_CAPACITY).
 * AQUA_ERR_IO: the file cannot be read.  AQUA_ERR_FORMAT: a line with
 * another number of fields, or a column with no number or out of its type's
 * range; *bad_line (if not NULL) = its 1-based line number. */
aqua_status aqua_read_fastascii(const char* path, uint32_t n_cols,
                                const int32_t* col_types, void* out,
                                uint64_t max_rows, uint64_t* n_rows,
                                uint64_t* bad_line);

/* Number of kernel launches one aqua_step() step issues (for accounting). */
uint32_t aqua_launches_per_step(aqua_ctx* ctx);

#ifdef __cplusplus
}
#endif

#endif
