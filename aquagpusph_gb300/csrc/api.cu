// C ABI of the aqua_gb300 library: context, device memory, step scheduling
// (CUDA graphs) and the reference-facing entry points.
//
// Ownership mirrors the reference's CalcServer (CalcServer.cpp:139-535,
// 566-569): the context owns every device buffer of the resident case (two
// sets of particle Variables that alternate between steps, plus the step
// scratch) and allocates them all at creation; steps allocate nothing.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>

#include "aqua_internal.cuh"
#include "kernels.cuh"

using namespace aqua;

namespace aqua {
// test-only switch of aqua_debug_fake_timeouts(): read when a step or a
// tensor-core kernel is enqueued (graphs keep the value they were captured
// with)
int g_debug_fake_timeout = 0;
}  // namespace aqua

namespace {
constexpr uint32_t kMaxCases = 4096;
}

struct aqua_ctx
{
    int device = 0;
    int dims = 3;
    uint32_t capacity = 0;  // max particles
    uint32_t ncap = 0;      // cell capacity
    uint32_t N = 0;
    uint32_t passes = 3;
    Consts consts{};
    VarSet set[2]{};
    int cur = 0;
    StepBufs b{};
    DevScalars* sc = nullptr;      // resident state scalars
    DevScalars* sc_aux = nullptr;  // standalone link-list / sort
    CaseScalars* cs = nullptr;     // per-case scalars (kMaxCases)
    CaseScalars* cs_aux = nullptr; // standalone link-list (1 case)
    CaseMotion* cm = nullptr;      // per-case motion (kMaxCases)
    uint32_t* offsets = nullptr;   // case offsets (kMaxCases + 1)
    uint32_t n_cases = 1;
    int has_motion = 0;
    uint32_t* ihoc_out = nullptr;  // ihoc export buffer (ncap)
    float* report = nullptr;       // report staging (kReportValues)
    int* fs_keys = nullptr;        // free-surface maxima (kMaxFsSensors)
    float* fs_out = nullptr;       // decoded free-surface elevations
    int extras = 0;
    int fast = 0;              // 1: -use_fast_math step kernels
    unsigned sweep_grid = 0;   // persistent sweep blocks
    int sweep_variant = kSweepClusteredDefault;  // launch shape of the sweep
                                                 // (aqua_set_tuning)
    int sms = 1;
    void* pool = nullptr;
    size_t pool_bytes = 0;
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t graph[2] = { nullptr, nullptr };
    // configuration the graphs were captured for (particles, cases, roll)
    uint32_t graph_n = 0, graph_cases = 0;
    int graph_motion = -1;
    // pinned staging areas of the small host -> device copies (case scalars,
    // motions, offsets): a ring of kStageRing for aqua_set_state and one for
    // aqua_set_cases; an area is reused once its event shows that the copies
    // that last read it executed, which with a ring of four is almost never
    // a wait (the host may run several calls ahead of the device)
    static constexpr int kStageRing = 4;
    uint8_t* stage[2][kStageRing] = {};
    cudaEvent_t stage_ev[2][kStageRing] = {};
    int stage_next[2] = { 0, 0 };  // the ring entry stage_begin hands out
    int stage_cur[2] = { 0, 0 };   // the entry in use, for stage_done
    // stage boundary events (recorded when profiling is on): before the
    // link-list, before the gather, before the sweep, after the sweep, end
    static constexpr int kEvents = 5;
    cudaEvent_t ev[kEvents] = {};
    int profiling = 0;
};

namespace {

#define AQ_CUDA(call)                                                          \
    do {                                                                       \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess) {                                               \
            std::fprintf(stderr, "aqua_gb300: %s failed: %s\n", #call,         \
                         cudaGetErrorString(e_));                              \
            return AQUA_ERR_CUDA;                                              \
        }                                                                      \
    } while (0)

struct Carver
{
    char* base;
    size_t off = 0;
    template<typename T>
    T* take(size_t count)
    {
        off = (off + 255) & ~(size_t)255;
        T* p = reinterpret_cast<T*>(base ? base + off : nullptr);
        off += count * sizeof(T);
        return p;
    }
};

aqua_status
build_consts(const aqua_params* p, Consts& c)
{
    if (!p || (p->dims != 2 && p->dims != 3) || p->n_sets == 0 ||
        p->n_sets > (uint32_t)kMaxSets || !p->refd || !p->visc_dyn ||
        !p->delta || !(p->h > 0.f) || !(p->support > 0.f) || !(p->H > 0.f))
        return AQUA_ERR_INVALID;
    if (p->boundary != AQUA_BOUNDARY_BIE && p->boundary != AQUA_BOUNDARY_BI)
        return AQUA_ERR_INVALID;
    if (p->scheme == AQUA_SCHEME_MIDPOINT) {
        if (p->iter_midpoint_max != 1)
            return AQUA_ERR_INVALID;  // one midpoint iteration (canonical stack)
    } else if (p->scheme == AQUA_SCHEME_IMPROVED_EULER) {
        // BIe/ElasticBounce.cl reads r_in and u_in by sorted index, which
        // under improved_euler.cl hold the predictor's unsorted output
        if (p->boundary != AQUA_BOUNDARY_BI)
            return AQUA_ERR_INVALID;
    } else {
        return AQUA_ERR_INVALID;
    }
    std::memset(&c, 0, sizeof(c));
    c.dims = p->dims;
    c.n_sets = p->n_sets;
    c.h = p->h;
    c.support = p->support;
    c.H = p->H;
    c.CONW = p->CONW;
    c.CONF = p->CONF;
    c.SUPPORT = p->SUPPORT;
    c.DIMS = p->DIMS;
    c.cs = p->cs;
    c.p0 = p->p0;
    std::memcpy(c.g, p->g, sizeof(c.g));
    c.courant = p->courant;
    c.dt_Ma = p->dt_Ma;
    c.dt_min = p->dt_min;
    c.dt_fixed = p->dt_fixed;
    std::memcpy(c.domain_min, p->domain_min, sizeof(c.domain_min));
    std::memcpy(c.domain_max, p->domain_max, sizeof(c.domain_max));
    c.dr_factor = p->dr_factor;
    c.min_bound_dist = p->min_bound_dist;
    c.relax_midpoint = p->relax_midpoint;
    c.iter_midpoint_max = p->iter_midpoint_max;
    c.boundary = p->boundary;
    c.scheme = p->scheme;
    for (uint32_t k = 0; k < p->n_sets; k++) {
        c.refd[k] = p->refd[k];
        c.visc_dyn[k] = p->visc_dyn[k];
        c.delta[k] = p->delta[k];
    }
    // LinkList.cpp:156 and LinkList.cl.in:73, both in float
    volatile float sh = p->support * p->h;
    c.cell_length = sh;
    c.idist = 1.f / sh;
    // |r_ij|^2 at or above this bound gives |r_ij| / H >= SUPPORT for sure;
    // pairs below it take the exact test
    const double lim = (double)p->SUPPORT * (double)p->H;
    c.q2_reject = (float)(lim * lim * (1.0 + 1.0e-4));
    c.inv_H = 1.f / p->H;
    c.w_conw = (p->dims == 3 ? WendlandC<3>::W : WendlandC<2>::W) * p->CONW;
    c.f_conf = (p->dims == 3 ? WendlandC<3>::F : WendlandC<2>::F) * p->CONF;
    c.f_over_w = c.f_conf / c.w_conw;
    return AQUA_OK;
}

uint32_t
cells_from_domain(const aqua_params* p)
{
    const float cl = p->support * p->h;
    unsigned long long n = 1;
    for (int k = 0; k < p->dims; k++) {
        const double span = (double)p->domain_max[k] - (double)p->domain_min[k];
        if (!(span > 0))
            return 0;
        n *= (unsigned long long)(span / cl) + 8ull;
    }
    return n > 0xffffffffull ? 0u : (uint32_t)n;
}

uint32_t
bits_for(uint32_t maxval)
{
    uint32_t b = 0;
    while (b < 32 && (1ull << b) <= maxval)
        b++;
    return b;
}

size_t
layout(aqua_ctx* x, char* base)
{
    Carver cv{ base };
    const uint32_t n = x->capacity;
    const int VS = (x->dims == 3) ? 4 : 2;
    for (int s = 0; s < 2; s++) {
        VarSet& v = x->set[s];
        v.cid = cv.take<uint32_t>(n);
        v.id = cv.take<uint32_t>(n);
        v.iset = cv.take<uint32_t>(n);
        v.imove = cv.take<int32_t>(n);
        v.r = cv.take<float>((size_t)n * VS);
        v.normal = cv.take<float>((size_t)n * VS);
        v.tangent = cv.take<float>((size_t)n * VS);
        v.binormal = cv.take<float>((size_t)n * VS);
        v.u = cv.take<float>((size_t)n * VS);
        v.dudt = cv.take<float>((size_t)n * VS);
        v.rho = cv.take<float>(n);
        v.drhodt = cv.take<float>(n);
        v.m = cv.take<float>(n);
        v.p = cv.take<float>(n);
    }
    StepBufs& b = x->b;
    for (int k = 0; k < 2; k++) {
        b.keys[k] = cv.take<uint32_t>(n);
        b.vals[k] = cv.take<uint32_t>(n);
    }
    b.sort_scratch = cv.take<uint32_t>(sort_scratch_words(n > 0 ? n : 1));
    b.cells = cv.take<uint2>(x->ncap);
    b.chunks = cv.take<uint2>(n);
    b.wall_range = cv.take<uint2>(x->ncap);
    b.id_sorted = cv.take<uint32_t>(n);
    b.r_in = cv.take<float>((size_t)n * VS);
    b.u_in = cv.take<float>((size_t)n * VS);
    b.dudt_in = cv.take<float>((size_t)n * VS);
    b.rho_in = cv.take<float>(n);
    b.drhodt_in = cv.take<float>(n);
    b.posq = cv.take<float4>(n);
    b.velq = cv.take<float4>(n);
    b.pmq = cv.take<float2>(n);
    b.grad_p = cv.take<float>((size_t)n * VS);
    b.lap_u = cv.take<float>((size_t)n * VS);
    b.div_u = cv.take<float>(n);
    b.lap_p = cv.take<float>(n);
    b.grad_w_bi = cv.take<float>((size_t)n * VS);
    b.div_u_bi = cv.take<float>(n);
    b.shepard = cv.take<float>(n);
    b.rec0 = cv.take<float4>(n);
    b.rec1 = cv.take<float4>(n);
    b.cell_mark = cv.take<uint8_t>(x->ncap);
    b.work = cv.take<uint2>(n);
    b.wcl = cv.take<uint4>(n);
    b.crow = cv.take<uint2>((size_t)9 * x->ncap);
    b.clu = cv.take<uint2>(n);
    b.cperm = cv.take<uint32_t>(n);
    x->sc = cv.take<DevScalars>(1);
    x->sc_aux = cv.take<DevScalars>(1);
    x->cs = cv.take<CaseScalars>(kMaxCases);
    x->cs_aux = cv.take<CaseScalars>(1);
    x->cm = cv.take<CaseMotion>(kMaxCases);
    x->offsets = cv.take<uint32_t>(kMaxCases + 1);
    x->ihoc_out = cv.take<uint32_t>(x->ncap);
    x->report = cv.take<float>(kReportValues);
    x->fs_keys = cv.take<int>(kMaxFsSensors);
    x->fs_out = cv.take<float>(kMaxFsSensors);
    return cv.off + 256;
}

void
drop_graphs(aqua_ctx* x)
{
    for (int k = 0; k < 2; k++) {
        if (x->graph[k])
            cudaGraphExecDestroy(x->graph[k]);
        x->graph[k] = nullptr;
    }
}

// Layout of the pinned staging area: the step scalars, then per-case
// scalars, motions and offsets for up to kMaxCases cases
constexpr size_t kStageCs = 256;
constexpr size_t kStageCm = kStageCs + ((kMaxCases * sizeof(CaseScalars) + 255) & ~(size_t)255);
constexpr size_t kStageOff = kStageCm + ((kMaxCases * sizeof(CaseMotion) + 255) & ~(size_t)255);
constexpr size_t kStageBytes = kStageOff + (kMaxCases + 1) * sizeof(uint32_t);

// Staging area `slot` for the next small copies: waits (if at all) for the
// copies that last read it, so that the host may overwrite it.  The copies
// themselves stay asynchronous; stage_done() marks their position in the
// stream.
constexpr int kStageState = 0;  // aqua_set_state
constexpr int kStageCases = 1;  // aqua_set_cases

uint8_t*
stage_begin(aqua_ctx* x, int slot)
{
    const int k = x->stage_next[slot];
    x->stage_cur[slot] = k;
    x->stage_next[slot] = (k + 1) % aqua_ctx::kStageRing;
    return cudaEventSynchronize(x->stage_ev[slot][k]) == cudaSuccess
               ? x->stage[slot][k]
               : nullptr;
}

cudaError_t
stage_done(aqua_ctx* x, int slot, cudaStream_t s)
{
    return cudaEventRecord(x->stage_ev[slot][x->stage_cur[slot]], s);
}

// The clustered sweep runs for the fast build in 3-D with BIe walls and the
// midpoint scheme when the chosen variant is a clustered one
bool
sweep_clustered(const aqua_ctx* x)
{
    return x->fast && x->dims == 3 && x->sweep_variant >= kSweepClustered &&
           x->consts.boundary == AQUA_BOUNDARY_BIE &&
           x->consts.scheme == AQUA_SCHEME_MIDPOINT &&
           x->consts.SUPPORT == 2.f;  // the Wendland support
}

// Launches one step on `s` (the resident state advances from set[cur] to
// set[cur ^ 1]; the caller flips cur).
aqua_status
enqueue_step(aqua_ctx* x, int cur, cudaStream_t s)
{
    const VarSet& S = x->set[cur];
    const VarSet& T = x->set[cur ^ 1];
    StepBufs& b = x->b;
    const uint32_t N = x->N;
    if (x->profiling)
        AQ_CUDA(cudaEventRecordWithFlags(x->ev[0], s, cudaEventRecordExternal));
    AQ_CUDA(launch_begin(x->sc, x->cs, x->n_cases, b.cells, b.wall_range,
                         x->consts.sample_on ? b.cell_mark : nullptr, x->ncap,
                         N, s));
    // one case: every particle's case id is 0 (not read)
    const uint32_t* cid = x->n_cases > 1 ? S.cid : nullptr;
    if (x->dims == 3) {
        AQ_CUDA(launch_minmax<3>(x->consts, S.r, S.imove, cid, N, x->cs,
                                 x->sc, s));
        AQ_CUDA(launch_ncells<3>(x->consts, x->cs, x->n_cases, x->sc, x->ncap, s));
        AQ_CUDA(launch_icell_hist<3>(x->consts, S.r, S.imove, cid, N, x->cs,
                                     x->sc, b.keys[0], b.sort_scratch,
                                     x->passes, s));
    } else {
        AQ_CUDA(launch_minmax<2>(x->consts, S.r, S.imove, cid, N, x->cs,
                                 x->sc, s));
        AQ_CUDA(launch_ncells<2>(x->consts, x->cs, x->n_cases, x->sc, x->ncap, s));
        AQ_CUDA(launch_icell_hist<2>(x->consts, S.r, S.imove, cid, N, x->cs,
                                     x->sc, b.keys[0], b.sort_scratch,
                                     x->passes, s));
    }
    AQ_CUDA(launch_radix_passes(b.keys, b.vals, N, x->passes, b.sort_scratch,
                                true, x->sc, s));
    StepArgs a;
    a.N = N;
    a.ncap = x->ncap;
    a.src = S;
    a.dst = T;
    a.b = b;
    a.skeys = b.keys[x->passes & 1];
    a.perm = b.vals[x->passes & 1];
    a.sc = x->sc;
    a.cs = x->cs;
    a.cm = x->cm;
    a.n_cases = x->n_cases;
    a.extras = x->extras;
    const bool clustered = sweep_clustered(x);
    a.clustered = clustered ? 1 : 0;
    Consts cst = x->consts;
    cst.debug_fake_timeout = g_debug_fake_timeout ? 1u : 0u;
    if (x->profiling)
        AQ_CUDA(cudaEventRecordWithFlags(x->ev[1], s, cudaEventRecordExternal));
    if (x->dims == 3)
        AQ_CUDA(launch_gather<3>(x->fast, x->consts, a, s));
    else
        AQ_CUDA(launch_gather<2>(x->fast, x->consts, a, s));
    if (x->consts.boundary == AQUA_BOUNDARY_BI) {
        if (x->dims == 3)
            AQ_CUDA(launch_bi_walls<3>(x->fast, x->consts, a, s));
        else
            AQ_CUDA(launch_bi_walls<2>(x->fast, x->consts, a, s));
    }
    if (x->profiling)
        AQ_CUDA(cudaEventRecordWithFlags(x->ev[2], s, cudaEventRecordExternal));
    if (clustered) {
        AQ_CUDA(fast::launch_sweep_cl(cst, a, x->sweep_grid, x->sweep_variant,
                                      (unsigned)x->sms, s));
    } else {
        // a clustered choice where the clustered sweep does not apply falls
        // back to the direct sweep's untuned shape
        const bool cl_pick = x->sweep_variant >= kSweepClustered;
        const int v = cl_pick ? 9 : x->sweep_variant;
        const unsigned g = cl_pick ? (unsigned)x->sms * 14u : x->sweep_grid;
        if (x->dims == 3)
            AQ_CUDA(launch_sweep<3>(x->fast, cst, a, g, v, s));
        else
            AQ_CUDA(launch_sweep<2>(x->fast, cst, a, g, v, s));
    }
    if (x->profiling)
        AQ_CUDA(cudaEventRecordWithFlags(x->ev[3], s, cudaEventRecordExternal));
    AQ_CUDA(launch_finalize(x->sc, x->cs, x->cm, x->n_cases, s));
    if (x->has_motion) {
        if (x->dims == 3)
            AQ_CUDA(launch_motion<3>(a, s));
        else
            AQ_CUDA(launch_motion<2>(a, s));
    }
    if (x->profiling)
        AQ_CUDA(cudaEventRecordWithFlags(x->ev[4], s, cudaEventRecordExternal));
    return AQUA_OK;
}

aqua_status
copy_in(void* dst, const void* src, size_t bytes, int on_host, cudaStream_t s)
{
    if (!src)
        return AQUA_ERR_INVALID;
    AQ_CUDA(cudaMemcpyAsync(dst, src, bytes,
                            on_host ? cudaMemcpyHostToDevice
                                    : cudaMemcpyDeviceToDevice, s));
    return AQUA_OK;
}

aqua_status
copy_out(void* dst, const void* src, size_t bytes, int on_host, cudaStream_t s)
{
    if (!dst)
        return AQUA_OK;
    AQ_CUDA(cudaMemcpyAsync(dst, src, bytes,
                            on_host ? cudaMemcpyDeviceToHost
                                    : cudaMemcpyDeviceToDevice, s));
    return AQUA_OK;
}

#define AQ_TRY(expr)                                                           \
    do {                                                                       \
        aqua_status st_ = (expr);                                              \
        if (st_ != AQUA_OK)                                                    \
            return st_;                                                        \
    } while (0)

aqua_status
status_of(uint32_t err)
{
    if (err & kErrCapacity)
        return AQUA_ERR_CAPACITY;
    if (err & kErrNonFinite)
        return AQUA_ERR_NONFINITE;
    if (err & kErrDt)
        return AQUA_ERR_DT;
    if (err & kErrTimeout)
        return AQUA_ERR_TIMEOUT;
    return AQUA_OK;
}

}  // namespace

extern "C" {

const char*
aqua_version(void)
{
    return "aqua_gb300 0.1 (sm_103a)";
}

aqua_status
aqua_malloc(void** ptr, size_t bytes)
{
    if (!ptr || bytes == 0)
        return AQUA_ERR_INVALID;
    *ptr = nullptr;
    if (cudaMalloc(ptr, bytes) != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        return AQUA_ERR_NO_MEMORY;
    }
    return AQUA_OK;
}

aqua_status
aqua_free(void* ptr)
{
    if (ptr)
        AQ_CUDA(cudaFree(ptr));
    return AQUA_OK;
}

aqua_status
aqua_memcpy(void* dst, const void* src, size_t bytes, int kind)
{
    if ((!dst || !src) && bytes)
        return AQUA_ERR_INVALID;
    cudaMemcpyKind k;
    switch (kind) {
    case AQUA_COPY_H2D: k = cudaMemcpyHostToDevice; break;
    case AQUA_COPY_D2H: k = cudaMemcpyDeviceToHost; break;
    case AQUA_COPY_D2D: k = cudaMemcpyDeviceToDevice; break;
    default: return AQUA_ERR_INVALID;
    }
    if (bytes)
        AQ_CUDA(cudaMemcpy(dst, src, bytes, k));
    return AQUA_OK;
}

aqua_status
aqua_create(const aqua_params* params, uint32_t capacity,
            uint32_t ihoc_capacity, aqua_ctx** out)
{
    if (!out || capacity == 0)
        return AQUA_ERR_INVALID;
    *out = nullptr;
    Consts c{};
    AQ_TRY(build_consts(params, c));
    aqua_ctx* x = new (std::nothrow) aqua_ctx();
    if (!x)
        return AQUA_ERR_NO_MEMORY;
    x->consts = c;
    x->dims = params->dims;
    x->capacity = capacity;
    x->ncap = ihoc_capacity ? ihoc_capacity : cells_from_domain(params);
    if (x->ncap == 0) {
        delete x;
        return AQUA_ERR_INVALID;
    }
    x->passes = sort_passes(bits_for(x->ncap));
    int sms = 0;
    if (cudaGetDevice(&x->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount,
                               x->device) != cudaSuccess) {
        delete x;
        return AQUA_ERR_CUDA;
    }
    x->sms = sms > 0 ? sms : 1;
    // untuned default: the clustered sweep (fast 3-D BIe midpoint) with 3
    // blocks of 8 warps per SM; elsewhere the direct sweep with prefetch at
    // 28 warps per SM (see enqueue_step)
    x->sweep_grid = (unsigned)x->sms * kSweepClusteredBlocks;
    if (fast::prepare_sweep_cl() != cudaSuccess) {
        delete x;
        return AQUA_ERR_CUDA;
    }
    x->pool_bytes = layout(x, nullptr);
    if (cudaMalloc(&x->pool, x->pool_bytes) != cudaSuccess) {
        cudaGetLastError();
        delete x;
        return AQUA_ERR_NO_MEMORY;
    }
    layout(x, (char*)x->pool);
    for (int k = 0; k < aqua_ctx::kEvents; k++)
        if (cudaEventCreate(&x->ev[k]) != cudaSuccess) {
            cudaFree(x->pool);
            delete x;
            return AQUA_ERR_CUDA;
        }
    bool ok = cudaMemset(x->pool, 0, x->pool_bytes) == cudaSuccess &&
              cudaStreamCreateWithFlags(&x->cap_stream, cudaStreamNonBlocking) ==
                  cudaSuccess;
    for (int k = 0; ok && k < 2; k++)
        for (int q = 0; ok && q < aqua_ctx::kStageRing; q++)
            ok = cudaMallocHost(&x->stage[k][q], kStageBytes) == cudaSuccess &&
                 cudaEventCreateWithFlags(&x->stage_ev[k][q],
                                          cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        aqua_destroy(x);
        return AQUA_ERR_CUDA;
    }
    *out = x;
    return AQUA_OK;
}

aqua_status
aqua_destroy(aqua_ctx* x)
{
    if (!x)
        return AQUA_ERR_INVALID;
    drop_graphs(x);
    if (x->cap_stream)
        cudaStreamDestroy(x->cap_stream);
    for (int k = 0; k < aqua_ctx::kEvents; k++)
        if (x->ev[k])
            cudaEventDestroy(x->ev[k]);
    for (int k = 0; k < 2; k++)
        for (int q = 0; q < aqua_ctx::kStageRing; q++) {
            if (x->stage_ev[k][q]) {
                cudaEventSynchronize(x->stage_ev[k][q]);  // no copy still reads it
                cudaEventDestroy(x->stage_ev[k][q]);
            }
            if (x->stage[k][q])
                cudaFreeHost(x->stage[k][q]);
        }
    if (x->pool)
        cudaFree(x->pool);
    delete x;
    return AQUA_OK;
}

aqua_status
aqua_set_params(aqua_ctx* x, const aqua_params* params)
{
    if (!x || !params || params->dims != x->dims)
        return AQUA_ERR_INVALID;
    Consts c{};
    AQ_TRY(build_consts(params, c));
    // the rate sample is a setting of the context, not of the parameters
    c.sample_on = x->consts.sample_on;
    c.sample_thr = x->consts.sample_thr;
    c.sample_seed = x->consts.sample_seed;
    x->consts = c;
    drop_graphs(x);
    return AQUA_OK;
}

aqua_status
aqua_set_extras(aqua_ctx* x, int on)
{
    if (!x)
        return AQUA_ERR_INVALID;
    x->extras = on ? 1 : 0;
    drop_graphs(x);
    return AQUA_OK;
}

aqua_status
aqua_set_precision(aqua_ctx* x, int mode)
{
    if (!x || (mode != AQUA_PRECISION_EXACT && mode != AQUA_PRECISION_FAST))
        return AQUA_ERR_INVALID;
    x->fast = (mode == AQUA_PRECISION_FAST) ? 1 : 0;
    drop_graphs(x);
    return AQUA_OK;
}

aqua_status
aqua_set_tuning(aqua_ctx* x, uint32_t sweep_variant, uint32_t blocks_per_sm)
{
    if (!x || sweep_variant >= (uint32_t)kSweepVariants || blocks_per_sm == 0 ||
        blocks_per_sm > 32)
        return AQUA_ERR_INVALID;
    x->sweep_variant = (int)sweep_variant;
    x->sweep_grid = (unsigned)x->sms * blocks_per_sm;
    drop_graphs(x);
    return AQUA_OK;
}

aqua_status
aqua_set_state(aqua_ctx* x, uint32_t N, const aqua_vars* v, int on_host,
               float t, float dt, uint32_t iter, void* stream)
{
    if (!x || !v || N == 0 || N > x->capacity)
        return AQUA_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t VS = (x->dims == 3) ? 4 : 2;
    VarSet& d = x->set[x->cur];
    AQ_TRY(copy_in(d.id, v->id, N * 4ull, on_host, s));
    AQ_TRY(copy_in(d.iset, v->iset, N * 4ull, on_host, s));
    AQ_TRY(copy_in(d.imove, v->imove, N * 4ull, on_host, s));
    AQ_TRY(copy_in(d.r, v->r, N * VS * 4, on_host, s));
    AQ_TRY(copy_in(d.normal, v->normal, N * VS * 4, on_host, s));
    AQ_TRY(copy_in(d.tangent, v->tangent, N * VS * 4, on_host, s));
    if (v->binormal)
        AQ_TRY(copy_in(d.binormal, v->binormal, N * VS * 4, on_host, s));
    AQ_TRY(copy_in(d.u, v->u, N * VS * 4, on_host, s));
    AQ_TRY(copy_in(d.dudt, v->dudt, N * VS * 4, on_host, s));
    AQ_TRY(copy_in(d.rho, v->rho, N * 4ull, on_host, s));
    AQ_TRY(copy_in(d.drhodt, v->drhodt, N * 4ull, on_host, s));
    AQ_TRY(copy_in(d.m, v->m, N * 4ull, on_host, s));
    AQ_TRY(copy_in(d.p, v->p, N * 4ull, on_host, s));
    x->N = N;
    // the step scalars and one case holding every particle (aqua_set_cases()
    // splits them), through the pinned staging area: asynchronous
    uint8_t* st = stage_begin(x, kStageState);
    if (!st)
        return AQUA_ERR_CUDA;
    DevScalars* hs = reinterpret_cast<DevScalars*>(st);
    CaseScalars* c0 = reinterpret_cast<CaseScalars*>(st + kStageCs);
    CaseMotion* m0 = reinterpret_cast<CaseMotion*>(st + kStageCm);
    uint32_t* off = reinterpret_cast<uint32_t*>(st + kStageOff);
    std::memset(hs, 0, sizeof(*hs));
    std::memset(c0, 0, sizeof(*c0));
    c0->t = t;
    c0->dt = dt;
    c0->iter = iter;
    c0->dt_next = 0x7f800000u;
    c0->cos_psi = c0->cos_psi_in = 1.f;
    std::memset(m0, 0, sizeof(*m0));
    off[0] = 0u;
    off[1] = N;
    x->n_cases = 1;
    x->has_motion = 0;
    AQ_CUDA(cudaMemcpyAsync(x->sc, hs, sizeof(*hs), cudaMemcpyHostToDevice, s));
    AQ_CUDA(cudaMemcpyAsync(x->cs, c0, sizeof(*c0), cudaMemcpyHostToDevice, s));
    AQ_CUDA(cudaMemcpyAsync(x->cm, m0, sizeof(*m0), cudaMemcpyHostToDevice, s));
    AQ_CUDA(cudaMemcpyAsync(x->offsets, off, 2 * sizeof(uint32_t),
                            cudaMemcpyHostToDevice, s));
    AQ_CUDA(stage_done(x, kStageState, s));
    AQ_CUDA(launch_set_case_ids(x->set[x->cur].cid, x->offsets, 1, N, s));
    return AQUA_OK;
}

aqua_status
aqua_get_state(aqua_ctx* x, aqua_vars* v, int on_host, void* stream)
{
    if (!x || !v || x->N == 0)
        return AQUA_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t N = x->N, VS = (x->dims == 3) ? 4 : 2;
    const VarSet& d = x->set[x->cur];
    AQ_TRY(copy_out(v->id, d.id, N * 4, on_host, s));
    AQ_TRY(copy_out(v->iset, d.iset, N * 4, on_host, s));
    AQ_TRY(copy_out(v->imove, d.imove, N * 4, on_host, s));
    AQ_TRY(copy_out(v->r, d.r, N * VS * 4, on_host, s));
    AQ_TRY(copy_out(v->normal, d.normal, N * VS * 4, on_host, s));
    AQ_TRY(copy_out(v->tangent, d.tangent, N * VS * 4, on_host, s));
    AQ_TRY(copy_out(v->binormal, d.binormal, N * VS * 4, on_host, s));
    AQ_TRY(copy_out(v->u, d.u, N * VS * 4, on_host, s));
    AQ_TRY(copy_out(v->dudt, d.dudt, N * VS * 4, on_host, s));
    AQ_TRY(copy_out(v->rho, d.rho, N * 4, on_host, s));
    AQ_TRY(copy_out(v->drhodt, d.drhodt, N * 4, on_host, s));
    AQ_TRY(copy_out(v->m, d.m, N * 4, on_host, s));
    AQ_TRY(copy_out(v->p, d.p, N * 4, on_host, s));
    AQ_TRY(copy_out(v->shepard, x->b.shepard, N * 4, on_host, s));
    return AQUA_OK;
}

aqua_status
aqua_get_extra(aqua_ctx* x, aqua_extra* e, int on_host, void* stream)
{
    if (!x || !e || x->N == 0)
        return AQUA_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t N = x->N, VS = (x->dims == 3) ? 4 : 2;
    const StepBufs& b = x->b;
    AQ_TRY(copy_out(e->r_in, b.r_in, N * VS * 4, on_host, s));
    AQ_TRY(copy_out(e->u_in, b.u_in, N * VS * 4, on_host, s));
    AQ_TRY(copy_out(e->dudt_in, b.dudt_in, N * VS * 4, on_host, s));
    AQ_TRY(copy_out(e->rho_in, b.rho_in, N * 4, on_host, s));
    AQ_TRY(copy_out(e->drhodt_in, b.drhodt_in, N * 4, on_host, s));
    AQ_TRY(copy_out(e->icell, b.keys[x->passes & 1], N * 4, on_host, s));
    AQ_TRY(copy_out(e->id_unsorted, b.vals[x->passes & 1], N * 4, on_host, s));
    AQ_TRY(copy_out(e->id_sorted, b.id_sorted, N * 4, on_host, s));
    if (e->ihoc) {
        AQ_CUDA(launch_export_ihoc(b.cells, x->ihoc_out, x->ncap, x->sc, s));
        AQ_TRY(copy_out(e->ihoc, x->ihoc_out, (size_t)x->ncap * 4, on_host, s));
    }
    AQ_TRY(copy_out(e->grad_p, b.grad_p, N * VS * 4, on_host, s));
    AQ_TRY(copy_out(e->lap_u, b.lap_u, N * VS * 4, on_host, s));
    AQ_TRY(copy_out(e->div_u, b.div_u, N * 4, on_host, s));
    AQ_TRY(copy_out(e->lap_p, b.lap_p, N * 4, on_host, s));
    AQ_TRY(copy_out(e->grad_w_bi, b.grad_w_bi, N * VS * 4, on_host, s));
    AQ_TRY(copy_out(e->div_u_bi, b.div_u_bi, N * 4, on_host, s));
    return AQUA_OK;
}

aqua_status
aqua_get_unsorted(aqua_ctx* x, int field, uint32_t first, uint32_t n,
                  void* out, int on_host, void* stream)
{
    if (!x || !out || n == 0 || x->N == 0 || first > x->N || n > x->N - first)
        return AQUA_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t VS = (x->dims == 3) ? 4 : 2;
    const VarSet& d = x->set[x->cur];
    const float* src = nullptr;
    uint32_t nc = 1;
    switch (field) {
    case AQUA_FIELD_R: src = d.r; nc = VS; break;
    case AQUA_FIELD_NORMAL: src = d.normal; nc = VS; break;
    case AQUA_FIELD_TANGENT: src = d.tangent; nc = VS; break;
    case AQUA_FIELD_U: src = d.u; nc = VS; break;
    case AQUA_FIELD_DUDT: src = d.dudt; nc = VS; break;
    case AQUA_FIELD_RHO: src = d.rho; break;
    case AQUA_FIELD_DRHODT: src = d.drhodt; break;
    case AQUA_FIELD_M: src = d.m; break;
    case AQUA_FIELD_P: src = d.p; break;
    case AQUA_FIELD_SHEPARD: src = x->b.shepard; break;
    case AQUA_FIELD_IMOVE: break;
    default: return AQUA_ERR_INVALID;
    }
    const size_t values = (size_t)n * nc;
    if (on_host && values > kReportValues)
        return AQUA_ERR_CAPACITY;
    float* dst = on_host ? x->report : (float*)out;
    if (field == AQUA_FIELD_IMOVE)
        AQ_CUDA(launch_unsorted_int(d.id, d.imove, x->N, first, n, dst, s));
    else
        AQ_CUDA(launch_unsorted(d.id, src, nc, x->N, first, n, dst, s));
    if (on_host) {
        AQ_CUDA(cudaMemcpyAsync(out, x->report, values * 4,
                                cudaMemcpyDeviceToHost, s));
        AQ_CUDA(cudaStreamSynchronize(s));
    }
    return AQUA_OK;
}

aqua_status
aqua_free_surface(aqua_ctx* x, const float* sensors, uint32_t n_sensors,
                  float dr, int32_t case_index, float* out, void* stream)
{
    if (!x || !sensors || !out || n_sensors == 0 ||
        n_sensors > kMaxFsSensors || x->N == 0 || !(dr > 0.f) ||
        (case_index >= 0 && (uint32_t)case_index >= x->n_cases))
        return AQUA_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    FreeSurfaceSensors fs;
    std::memset(&fs, 0, sizeof(fs));
    for (uint32_t k = 0; k < n_sensors; k++) {
        fs.xy[k][0] = sensors[2 * k];
        fs.xy[k][1] = sensors[2 * k + 1];
    }
    const VarSet& d = x->set[x->cur];
    AQ_CUDA(launch_free_surface(x->dims, d.r, d.imove, d.cid, case_index, x->N,
                                fs, n_sensors, dr, x->fs_keys, x->fs_out, s));
    AQ_CUDA(cudaMemcpyAsync(out, x->fs_out, n_sensors * 4ull,
                            cudaMemcpyDeviceToHost, s));
    AQ_CUDA(cudaStreamSynchronize(s));
    return AQUA_OK;
}

aqua_status
aqua_get_case_scalars(aqua_ctx* x, uint32_t first, uint32_t count,
                      aqua_scalars* out, void* stream)
{
    if (!x || !out || first + count > x->n_cases)
        return AQUA_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    CaseScalars* h = new (std::nothrow) CaseScalars[count ? count : 1];
    if (!h)
        return AQUA_ERR_NO_MEMORY;
    cudaError_t e = cudaMemcpyAsync(h, x->cs + first, count * sizeof(CaseScalars),
                                    cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        delete[] h;
        std::fprintf(stderr, "aqua_gb300: reading case scalars failed: %s\n",
                     cudaGetErrorString(e));
        return AQUA_ERR_CUDA;
    }
    for (uint32_t k = 0; k < count; k++) {
        out[k].t = h[k].t;
        out[k].dt = h[k].dt;
        out[k].iter = h[k].iter;
        std::memcpy(out[k].n_cells, h[k].n_cells, sizeof(out[k].n_cells));
        std::memcpy(out[k].r_min, h[k].r_min, sizeof(out[k].r_min));
        std::memcpy(out[k].r_max, h[k].r_max, sizeof(out[k].r_max));
    }
    delete[] h;
    return AQUA_OK;
}

aqua_status
aqua_set_cases(aqua_ctx* x, uint32_t n_cases, const uint32_t* offsets,
               const aqua_case* cases, void* stream)
{
    if (!x || !offsets || !cases || n_cases == 0 || n_cases > kMaxCases ||
        offsets[0] != 0 || offsets[n_cases] != x->N)
        return AQUA_ERR_INVALID;
    for (uint32_t k = 0; k < n_cases; k++)
        if (offsets[k + 1] < offsets[k])
            return AQUA_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    // the per-case records are built in the pinned staging area and copied
    // asynchronously
    uint8_t* st = stage_begin(x, kStageCases);
    if (!st)
        return AQUA_ERR_CUDA;
    CaseScalars* hs = reinterpret_cast<CaseScalars*>(st + kStageCs);
    CaseMotion* hm = reinterpret_cast<CaseMotion*>(st + kStageCm);
    uint32_t* ho = reinterpret_cast<uint32_t*>(st + kStageOff);
    int motion = 0;
    for (uint32_t k = 0; k < n_cases; k++) {
        std::memset(&hs[k], 0, sizeof(CaseScalars));
        std::memset(&hm[k], 0, sizeof(CaseMotion));
        hs[k].t = cases[k].t;
        hs[k].dt = cases[k].dt;
        hs[k].iter = cases[k].iter;
        hs[k].dt_next = 0x7f800000u;
        hm[k].enabled = cases[k].roll_enabled ? 1 : 0;
        hm[k].iset = cases[k].roll_iset;
        hm[k].amplitude = cases[k].roll_amplitude;
        hm[k].angular_freq = cases[k].roll_angular_freq;
        std::memcpy(hm[k].center, cases[k].roll_center, sizeof(hm[k].center));
        // the roll angle the boundary currently sits at: psi(t)
        const double w = cases[k].roll_angular_freq;
        const double A = cases[k].roll_amplitude;
        const double psi = hm[k].enabled ? A * std::sin(w * (double)cases[k].t) : 0.0;
        hs[k].psi = (float)psi;
        hs[k].psi_in = hs[k].psi;
        hs[k].omega = hm[k].enabled ? (float)(A * w * std::cos(w * (double)cases[k].t)) : 0.f;
        hs[k].cos_psi = (float)std::cos((double)hs[k].psi);
        hs[k].sin_psi = (float)std::sin((double)hs[k].psi);
        hs[k].cos_psi_in = hs[k].cos_psi;
        hs[k].sin_psi_in = hs[k].sin_psi;
        motion |= hm[k].enabled;
    }
    std::memcpy(ho, offsets, (n_cases + 1) * sizeof(uint32_t));
    cudaError_t e = cudaMemcpyAsync(x->cs, hs, n_cases * sizeof(CaseScalars),
                                    cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(x->cm, hm, n_cases * sizeof(CaseMotion),
                            cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(x->offsets, ho, (n_cases + 1) * sizeof(uint32_t),
                            cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = stage_done(x, kStageCases, s);
    if (e == cudaSuccess)
        e = launch_set_case_ids(x->set[x->cur].cid, x->offsets, n_cases, x->N, s);
    if (e != cudaSuccess) {
        std::fprintf(stderr, "aqua_gb300: aqua_set_cases failed: %s\n",
                     cudaGetErrorString(e));
        return AQUA_ERR_CUDA;
    }
    x->n_cases = n_cases;
    x->has_motion = motion;
    return AQUA_OK;
}

aqua_status
aqua_get_scalars(aqua_ctx* x, aqua_scalars* out, void* stream)
{
    if (!x || !out)
        return AQUA_ERR_INVALID;
    return aqua_get_case_scalars(x, 0, 1, out, stream);
}

aqua_status
aqua_step(aqua_ctx* x, uint32_t nsteps, int use_graph, void* stream)
{
    if (!x || x->N == 0)
        return AQUA_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    if (use_graph && (x->graph_n != x->N || x->graph_cases != x->n_cases ||
                      x->graph_motion != x->has_motion)) {
        // the launches depend on these: capture again
        drop_graphs(x);
        x->graph_n = x->N;
        x->graph_cases = x->n_cases;
        x->graph_motion = x->has_motion;
    }
    for (uint32_t k = 0; k < nsteps; k++) {
        if (!use_graph) {
            AQ_TRY(enqueue_step(x, x->cur, s));
        } else {
            cudaGraphExec_t& g = x->graph[x->cur];
            if (!g) {
                cudaGraph_t graph = nullptr;
                AQ_CUDA(cudaStreamBeginCapture(x->cap_stream,
                                               cudaStreamCaptureModeThreadLocal));
                aqua_status st = enqueue_step(x, x->cur, x->cap_stream);
                cudaError_t e = cudaStreamEndCapture(x->cap_stream, &graph);
                if (st != AQUA_OK) {
                    if (graph)
                        cudaGraphDestroy(graph);
                    return st;
                }
                AQ_CUDA(e);
                e = cudaGraphInstantiate(&g, graph, 0);
                cudaGraphDestroy(graph);
                AQ_CUDA(e);
            }
            AQ_CUDA(cudaGraphLaunch(g, s));
        }
        x->cur ^= 1;
    }
    return AQUA_OK;
}

aqua_status
aqua_check(aqua_ctx* x, void* stream)
{
    if (!x)
        return AQUA_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t err[2] = { 0, 0 };
    AQ_CUDA(cudaMemcpyAsync(&err[0], &x->sc->err, 4, cudaMemcpyDeviceToHost, s));
    AQ_CUDA(cudaMemcpyAsync(&err[1], &x->sc_aux->err, 4, cudaMemcpyDeviceToHost, s));
    AQ_CUDA(cudaStreamSynchronize(s));
    AQ_CUDA(cudaGetLastError());
    if (err[0] || err[1]) {
        const uint32_t zero = 0;
        AQ_CUDA(cudaMemcpyAsync(&x->sc->err, &zero, 4, cudaMemcpyHostToDevice, s));
        AQ_CUDA(cudaMemcpyAsync(&x->sc_aux->err, &zero, 4, cudaMemcpyHostToDevice, s));
        AQ_CUDA(cudaStreamSynchronize(s));
    }
    return status_of(err[0] | err[1]);
}

aqua_status
aqua_radix_sort(aqua_ctx* x, uint32_t* keys, uint32_t* perm, uint32_t* inv_perm,
                uint32_t n, uint32_t key_bits, void* stream)
{
    if (!x || !keys || n > x->capacity || key_bits > 32)
        return AQUA_ERR_INVALID;
    if (n == 0)
        return AQUA_OK;
    cudaStream_t s = (cudaStream_t)stream;
    StepBufs& b = x->b;
    const uint32_t passes = sort_passes(key_bits);
    AQ_CUDA(cudaMemcpyAsync(b.keys[0], keys, n * 4ull, cudaMemcpyDeviceToDevice, s));
    AQ_CUDA(launch_radix_passes(b.keys, b.vals, n, passes, b.sort_scratch,
                                false, x->sc_aux, s));
    const int r = passes & 1;
    AQ_CUDA(cudaMemcpyAsync(keys, b.keys[r], n * 4ull, cudaMemcpyDeviceToDevice, s));
    if (perm)
        AQ_CUDA(cudaMemcpyAsync(perm, b.vals[r], n * 4ull, cudaMemcpyDeviceToDevice, s));
    if (inv_perm)
        AQ_CUDA(launch_inverse_perm(b.vals[r], inv_perm, n, nullptr, s));
    return AQUA_OK;
}

aqua_status
aqua_linklist(aqua_ctx* x, const float* r_in, uint32_t N, uint32_t* icell,
              uint32_t* id_sorted, uint32_t* id_unsorted, uint32_t* ihoc,
              uint32_t ihoc_capacity, uint32_t* n_cells_host,
              float* r_min_host, float* r_max_host, void* stream)
{
    if (!x || !r_in || N == 0 || N > x->capacity || !icell || !ihoc ||
        ihoc_capacity == 0)
        return AQUA_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    StepBufs& b = x->b;
    const uint32_t ncap = ihoc_capacity < x->ncap ? ihoc_capacity : x->ncap;
    const uint32_t passes = sort_passes(bits_for(ncap));
    DevScalars hs;
    std::memset(&hs, 0, sizeof(hs));
    AQ_CUDA(cudaMemcpyAsync(x->sc_aux, &hs, sizeof(hs), cudaMemcpyHostToDevice, s));
    AQ_CUDA(launch_begin(x->sc_aux, x->cs_aux, 1, b.cells, b.wall_range,
                         nullptr, 0, N, s));
    if (x->dims == 3) {
        AQ_CUDA(launch_minmax<3>(x->consts, r_in, nullptr, nullptr, N, x->cs_aux,
                                 x->sc_aux, s));
        AQ_CUDA(launch_ncells<3>(x->consts, x->cs_aux, 1, x->sc_aux, ncap, s));
        AQ_CUDA(launch_icell_hist<3>(x->consts, r_in, nullptr, nullptr, N,
                                     x->cs_aux, x->sc_aux, b.keys[0],
                                     b.sort_scratch, passes, s));
    } else {
        AQ_CUDA(launch_minmax<2>(x->consts, r_in, nullptr, nullptr, N, x->cs_aux,
                                 x->sc_aux, s));
        AQ_CUDA(launch_ncells<2>(x->consts, x->cs_aux, 1, x->sc_aux, ncap, s));
        AQ_CUDA(launch_icell_hist<2>(x->consts, r_in, nullptr, nullptr, N,
                                     x->cs_aux, x->sc_aux, b.keys[0],
                                     b.sort_scratch, passes, s));
    }
    AQ_CUDA(launch_radix_passes(b.keys, b.vals, N, passes, b.sort_scratch,
                                true, x->sc_aux, s));
    const int r = passes & 1;
    AQ_CUDA(cudaMemcpyAsync(icell, b.keys[r], N * 4ull, cudaMemcpyDeviceToDevice, s));
    if (id_unsorted)
        AQ_CUDA(cudaMemcpyAsync(id_unsorted, b.vals[r], N * 4ull,
                                cudaMemcpyDeviceToDevice, s));
    if (id_sorted)
        AQ_CUDA(launch_inverse_perm(b.vals[r], id_sorted, N, x->sc_aux, s));
    AQ_CUDA(launch_ihoc(b.keys[r], N, ihoc, ncap, x->sc_aux, s));
    CaseScalars hc;
    AQ_CUDA(cudaMemcpyAsync(&hs, x->sc_aux, sizeof(hs), cudaMemcpyDeviceToHost, s));
    AQ_CUDA(cudaMemcpyAsync(&hc, x->cs_aux, sizeof(hc), cudaMemcpyDeviceToHost, s));
    AQ_CUDA(cudaStreamSynchronize(s));
    if (n_cells_host)
        std::memcpy(n_cells_host, hc.n_cells, sizeof(hc.n_cells));
    if (r_min_host)
        std::memcpy(r_min_host, hc.r_min, sizeof(hc.r_min));
    if (r_max_host)
        std::memcpy(r_max_host, hc.r_max, sizeof(hc.r_max));
    if (hs.err) {
        const uint32_t zero = 0;
        AQ_CUDA(cudaMemcpyAsync(&x->sc_aux->err, &zero, 4, cudaMemcpyHostToDevice, s));
        AQ_CUDA(cudaStreamSynchronize(s));
    }
    return status_of(hs.err);
}

aqua_status
aqua_set_profiling(aqua_ctx* x, int on)
{
    if (!x)
        return AQUA_ERR_INVALID;
    x->profiling = on ? 1 : 0;
    drop_graphs(x);
    return AQUA_OK;
}

aqua_status
aqua_stage_times(aqua_ctx* x, float* ms, uint32_t n)
{
    if (!x || !ms || n < 4 || !x->profiling)
        return AQUA_ERR_INVALID;
    AQ_CUDA(cudaEventSynchronize(x->ev[aqua_ctx::kEvents - 1]));
    for (int k = 0; k < 4; k++)
        AQ_CUDA(cudaEventElapsedTime(&ms[k], x->ev[k], x->ev[k + 1]));
    return AQUA_OK;
}

aqua_status
aqua_set_rate_sample(aqua_ctx* x, float fraction, uint32_t seed)
{
    if (!x || !(fraction > 0.f))
        return AQUA_ERR_INVALID;
    if (fraction >= 1.f) {
        x->consts.sample_on = 0;
    } else {
        x->consts.sample_on = 1;
        x->consts.sample_thr = (uint32_t)((double)fraction * 4294967296.0);
        x->consts.sample_seed = seed;
    }
    drop_graphs(x);
    return AQUA_OK;
}

aqua_status
aqua_debug_fake_timeouts(int on)
{
    g_debug_fake_timeout = on ? 1 : 0;
    return AQUA_OK;
}

uint32_t
aqua_launches_per_step(aqua_ctx* x)
{
    if (!x)
        return 0;
    // begin, minmax, ncells, icell+hist, (passes - 1) hist,
    // passes x (scan, scatter), gather, [BI walls,] chunks or (cell list,
    // clusters), sweep, finalize [, motion]
    return 4u + (x->passes - 1u) + 2u * x->passes + 4u +
           (sweep_clustered(x) ? 1u : 0u) +
           (x->consts.boundary == AQUA_BOUNDARY_BI ? 1u : 0u) +
           (x->has_motion ? 1u : 0u);
}

}  // extern "C"
