// The step kernels compiled with the reference's arithmetic (-fmad=false,
// IEEE division and square root): aqua::exact.  Also the mode-independent
// kernels of the step: the chunk list of the sweep, the end-of-step scalar
// update and the ihoc export.
#include "aqua_internal.cuh"
#include "kernels.cuh"

namespace aqua {

namespace exact {
#define AQUA_FAST_ARITH 0
#include "step_kernels.cuh"
#undef AQUA_FAST_ARITH
}  // namespace exact

namespace {

// Cell-aligned chunks of <= 32 sorted particles: s starts a chunk when it is
// 0, 32, 64, ... particles past the first particle of its cell.  One
// atomicAdd per block of 1024 reserves the block's chunks (in sorted order
// within the block), so the shared counter sees few atomics.
constexpr int kChunkThreads = 1024;
__global__ void __launch_bounds__(kChunkThreads)
k_chunks(const uint32_t* skeys, const uint2* cells, uint32_t N, uint2* chunks,
         DevScalars* sc)
{
    __shared__ uint32_t s_count[kChunkThreads / 32];
    if (sc->err)
        return;
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    bool start = false;
    uint2 w = make_uint2(0, 0);
    if (s < N) {
        const uint2 se = cells[skeys[s]];
        start = ((s - se.x) & 31u) == 0u;
        w = make_uint2(s, min(32u, se.y - s));
    }
    const unsigned b = __ballot_sync(0xffffffffu, start);
    if (lane == 0)
        s_count[warp] = __popc(b);
    __syncthreads();
    if (warp == 0) {
        // exclusive scan of the warps' counts, one reservation for the block
        const uint32_t v = lane < kChunkThreads / 32 ? s_count[lane] : 0u;
        uint32_t incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o)
                incl += t;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        uint32_t base = 0;
        if (lane == 0 && total)
            base = atomicAdd(&sc->n_chunks, total);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (lane < kChunkThreads / 32)
            s_count[lane] = base + incl - v;
    }
    __syncthreads();
    if (start)
        chunks[s_count[warp] + __popc(b & ((1u << lane) - 1u))] = w;
}

// End of step of every case: dt = min(dt_var) (Reduction tool), assert
// dt > 0, t += dt, iter += 1 (set_scalar tools); for a rolling case, the new
// roll angle and rate at the new time (the reference's motion tools run
// after the time step, cfd/motion.xml:59-71).
__global__ void
k_finalize(DevScalars* sc, CaseScalars* cs, const CaseMotion* cm,
           uint32_t n_cases)
{
    if (sc->err)
        return;
    for (uint32_t k = threadIdx.x; k < n_cases; k += blockDim.x) {
        CaseScalars& c = cs[k];
        const float dt = __uint_as_float(c.dt_next);
        if (!(dt > 0.f) || isinf(dt)) {
            atomicOr(&sc->err, kErrDt);
            continue;
        }
        c.dt = dt;
        c.t = (float)((double)c.t + (double)dt);
        c.iter = c.iter + 1;
        if (cm[k].enabled) {
            const double w = (double)cm[k].angular_freq;
            const double A = (double)cm[k].amplitude;
            const double psi = A * sin(w * (double)c.t);
            c.psi_in = c.psi;
            c.cos_psi_in = c.cos_psi;
            c.sin_psi_in = c.sin_psi;
            c.psi = (float)psi;
            c.omega = (float)(A * w * cos(w * (double)c.t));
            c.cos_psi = (float)cos((double)c.psi);
            c.sin_psi = (float)sin((double)c.psi);
        }
    }
}

// Prescribed roll of the boundary elements and probes of a moving case
// about `center` (z axis): un-transform with the previous angle, velocity
// from the new rate, transform with the new angle
// (cfd/Motions/UnTransform.cl, Velocity.cl, Transform.cl).
template<int D>
__global__ void __launch_bounds__(256)
k_motion(StepArgs a)
{
    constexpr int VS = Vec<D>::VS;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.N || a.sc->err)
        return;
    const VarSet& T = a.dst;
    const uint32_t k = T.cid[i];
    const CaseMotion& m = a.cm[k];
    if (!m.enabled || T.iset[i] != m.iset || T.imove[i] == 1)
        return;
    const CaseScalars& c = a.cs[k];
    float r[4], n[4], t[4];
    Vec<D>::load(T.r, i, r);
    Vec<D>::load(T.normal, i, n);
    Vec<D>::load(T.tangent, i, t);
    // un-transform (rotation by -psi_in about z, around the centre)
    for (int d = 0; d < VS; d++)
        r[d] = r[d] - m.center[d];
    const float ci = c.cos_psi_in, si = -c.sin_psi_in;
    float rl[4], nl[4], tl[4];
    for (int d = 0; d < 4; d++) {
        rl[d] = r[d];
        nl[d] = n[d];
        tl[d] = t[d];
    }
    rl[0] = ci * r[0] - si * r[1];
    rl[1] = si * r[0] + ci * r[1];
    nl[0] = ci * n[0] - si * n[1];
    nl[1] = si * n[0] + ci * n[1];
    tl[0] = ci * t[0] - si * t[1];
    tl[1] = si * t[0] + ci * t[1];
    // velocity of the rotation in the local frame, then rotated
    const float cp = c.cos_psi, sp = c.sin_psi;
    float ul[4] = { 0.f, 0.f, 0.f, 0.f }, u[4] = { 0.f, 0.f, 0.f, 0.f };
    ul[0] = -c.omega * rl[1];
    ul[1] = c.omega * rl[0];
    u[0] = cp * ul[0] - sp * ul[1];
    u[1] = sp * ul[0] + cp * ul[1];
    // transform with the new angle
    float ro[4], no[4], to[4];
    for (int d = 0; d < 4; d++) {
        ro[d] = rl[d];
        no[d] = nl[d];
        to[d] = tl[d];
    }
    ro[0] = cp * rl[0] - sp * rl[1];
    ro[1] = sp * rl[0] + cp * rl[1];
    no[0] = cp * nl[0] - sp * nl[1];
    no[1] = sp * nl[0] + cp * nl[1];
    to[0] = cp * tl[0] - sp * tl[1];
    to[1] = sp * tl[0] + cp * tl[1];
    for (int d = 0; d < VS; d++)
        ro[d] = ro[d] + m.center[d];
    float nn = 0.f, tt = 0.f;
    for (int d = 0; d < VS; d++) {
        nn = nn + no[d] * no[d];
        tt = tt + to[d] * to[d];
    }
    nn = sqrtf(nn);
    tt = sqrtf(tt);
    for (int d = 0; d < VS; d++) {
        no[d] = no[d] / nn;
        to[d] = to[d] / tt;
    }
    Vec<D>::store(T.r, i, ro);
    Vec<D>::store(T.normal, i, no);
    Vec<D>::store(T.tangent, i, to);
    Vec<D>::store(T.u, i, u);
}

// case id of every particle from the case offsets
__global__ void
k_set_case_ids(uint32_t* cid, const uint32_t* offsets, uint32_t n_cases,
               uint32_t N)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N)
        return;
    uint32_t lo = 0, hi = n_cases;  // offsets[lo] <= i < offsets[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) / 2;
        if (offsets[mid] <= i)
            lo = mid;
        else
            hi = mid;
    }
    cid[i] = lo;
}

__global__ void
k_export_ihoc(const uint2* cells, uint32_t* ihoc, uint32_t ncap,
              const DevScalars* sc)
{
    const uint32_t nw = sc->total_cells;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < ncap && c < nw;
         c += gridDim.x * blockDim.x)
        ihoc[c] = cells[c].x;
}

}  // namespace

template<int D>
cudaError_t
launch_gather(bool fast, const Consts& c, const StepArgs& a, cudaStream_t s)
{
    return fast ? fast::launch_gather_impl<D>(c, a, s)
                : exact::launch_gather_impl<D>(c, a, s);
}

template<int D>
cudaError_t
launch_sweep(bool fast, const Consts& c, const StepArgs& a, unsigned grid,
             int variant, cudaStream_t s)
{
    if (a.N) {
        k_chunks<<<(a.N + kChunkThreads - 1) / kChunkThreads, kChunkThreads, 0,
                   s>>>(a.skeys, a.b.cells, a.N, a.b.chunks, a.sc);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess)
            return e;
    }
    return fast ? fast::launch_sweep_impl<D>(c, a, grid, variant, s)
                : exact::launch_sweep_impl<D>(c, a, grid, variant, s);
}

template<int D>
cudaError_t
launch_bi_walls(bool fast, const Consts& c, const StepArgs& a, cudaStream_t s)
{
    return fast ? fast::launch_bi_walls_impl<D>(c, a, s)
                : exact::launch_bi_walls_impl<D>(c, a, s);
}

cudaError_t
launch_finalize(DevScalars* sc, CaseScalars* cs, const CaseMotion* cm,
                uint32_t n_cases, cudaStream_t s)
{
    k_finalize<<<1, 256, 0, s>>>(sc, cs, cm, n_cases);
    return cudaGetLastError();
}

template<int D>
cudaError_t
launch_motion(const StepArgs& a, cudaStream_t s)
{
    if (a.N == 0)
        return cudaSuccess;
    k_motion<D><<<(a.N + 255) / 256, 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t
launch_set_case_ids(uint32_t* cid, const uint32_t* offsets, uint32_t n_cases,
                    uint32_t N, cudaStream_t s)
{
    if (N == 0)
        return cudaSuccess;
    k_set_case_ids<<<(N + 255) / 256, 256, 0, s>>>(cid, offsets, n_cases, N);
    return cudaGetLastError();
}

cudaError_t
launch_export_ihoc(const uint2* cells, uint32_t* ihoc, uint32_t ncap,
                   const DevScalars* sc, cudaStream_t s)
{
    const unsigned g = min((ncap + 255u) / 256u, 152u * 8u);
    k_export_ihoc<<<g > 0 ? g : 1u, 256, 0, s>>>(cells, ihoc, ncap, sc);
    return cudaGetLastError();
}

template cudaError_t launch_bi_walls<2>(bool, const Consts&, const StepArgs&,
                                        cudaStream_t);
template cudaError_t launch_bi_walls<3>(bool, const Consts&, const StepArgs&,
                                        cudaStream_t);
template cudaError_t launch_motion<2>(const StepArgs&, cudaStream_t);
template cudaError_t launch_motion<3>(const StepArgs&, cudaStream_t);
template cudaError_t launch_gather<2>(bool, const Consts&, const StepArgs&, cudaStream_t);
template cudaError_t launch_gather<3>(bool, const Consts&, const StepArgs&, cudaStream_t);
template cudaError_t launch_sweep<2>(bool, const Consts&, const StepArgs&, unsigned,
                                     int, cudaStream_t);
template cudaError_t launch_sweep<3>(bool, const Consts&, const StepArgs&, unsigned,
                                     int, cudaStream_t);

}  // namespace aqua
