// The step kernels compiled with the reference's arithmetic (-fmad=false,
// IEEE division and square root): aqua::exact.  Also the mode-independent
// kernels of the step: the chunk list of the sweep, the end-of-step scalar
// update and the ihoc export.
#include "aqua_internal.cuh"
#include "kernels.cuh"

namespace aqua {

namespace exact {
#include "step_kernels.cuh"
}  // namespace exact

namespace {

// Cell-aligned chunks of <= 32 sorted particles: s starts a chunk when it is
// 0, 32, 64, ... particles past the first particle of its cell.
__global__ void __launch_bounds__(256)
k_chunks(const uint32_t* skeys, const uint2* cells, uint32_t N, uint2* chunks,
         DevScalars* sc)
{
    if (sc->err)
        return;
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    bool start = false;
    uint2 w = make_uint2(0, 0);
    if (s < N) {
        const uint2 se = cells[skeys[s]];
        start = ((s - se.x) & 31u) == 0u;
        w = make_uint2(s, min(32u, se.y - s));
    }
    const unsigned b = __ballot_sync(0xffffffffu, start);
    uint32_t base = 0;
    if (lane == 0 && b)
        base = atomicAdd(&sc->n_chunks, (uint32_t)__popc(b));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (start)
        chunks[base + __popc(b & ((1u << lane) - 1u))] = w;
}

__global__ void
k_finalize(DevScalars* sc)
{
    if (sc->err)
        return;
    const float dt = __uint_as_float(sc->dt_next);
    if (!(dt > 0.f) || isinf(dt)) {
        atomicOr(&sc->err, kErrDt);
        return;
    }
    sc->dt = dt;
    sc->t = (float)((double)sc->t + (double)dt);
    sc->iter = sc->iter + 1;
}

__global__ void
k_export_ihoc(const uint2* cells, uint32_t* ihoc, uint32_t ncap,
              const DevScalars* sc)
{
    const uint32_t nw = sc->n_cells[3];
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
             cudaStream_t s)
{
    if (a.N) {
        k_chunks<<<(a.N + 255) / 256, 256, 0, s>>>(a.skeys, a.b.cells, a.N,
                                                    a.b.chunks, a.sc);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess)
            return e;
    }
    return fast ? fast::launch_sweep_impl<D>(c, a, grid, s)
                : exact::launch_sweep_impl<D>(c, a, grid, s);
}

cudaError_t
launch_finalize(DevScalars* sc, cudaStream_t s)
{
    k_finalize<<<1, 1, 0, s>>>(sc);
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

template cudaError_t launch_gather<2>(bool, const Consts&, const StepArgs&, cudaStream_t);
template cudaError_t launch_gather<3>(bool, const Consts&, const StepArgs&, cudaStream_t);
template cudaError_t launch_sweep<2>(bool, const Consts&, const StepArgs&, unsigned,
                                     cudaStream_t);
template cudaError_t launch_sweep<3>(bool, const Consts&, const StepArgs&, unsigned,
                                     cudaStream_t);

}  // namespace aqua
