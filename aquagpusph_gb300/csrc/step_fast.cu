// The step kernels compiled with -use_fast_math (FMA contraction,
// approximate division and square root): aqua::fast.  Same source as the
// exact kernels (step_kernels.cuh); results stay within the 1e-5 relative
// tolerance of the reference's per-step rates (tests/test_gpu_fast.py).
// The fast build also has the clustered 3-D sweep (sweep_cl.cuh).
#include "aqua_internal.cuh"
#include "kernels.cuh"

namespace aqua {
namespace fast {
#define AQUA_FAST_ARITH 1
#include "step_kernels.cuh"
#include "sweep_cl.cuh"
#undef AQUA_FAST_ARITH

namespace {

template<int NW, int CAP, int MINB>
cudaError_t
launch_cl(const Consts& c, const StepArgs& a, unsigned grid, unsigned sms,
          cudaStream_t s)
{
    constexpr uint32_t kPer = kCellListThreads * kCellListItems;
    k_cell_list<<<max(1u, (a.N + kPer - 1) / kPer), kCellListThreads, 0, s>>>(
        a.skeys, a.N, a.b.cells, a.dst.cid, a.b.work, a.b.wcl, a.sc);
    k_clusters<<<sms * 8u, 256, 0, s>>>(c, a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    k_sweep_cl<NW, CAP, MINB><<<grid, NW * 32, sizeof(ClSmem<NW, CAP>), s>>>(c, a);
    return cudaGetLastError();
}

template<int NW, int CAP, int MINB>
cudaError_t
prepare_cl()
{
    return cudaFuncSetAttribute(k_sweep_cl<NW, CAP, MINB>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)sizeof(ClSmem<NW, CAP>));
}

}  // namespace

cudaError_t
launch_sweep_cl(const Consts& c, const StepArgs& a, unsigned grid, int variant,
                unsigned sms, cudaStream_t s)
{
    if (a.N == 0)
        return cudaSuccess;
    switch (variant) {
    case kSweepClustered + 0:
        return launch_cl<8, 2048, 2>(c, a, grid, sms, s);
    case kSweepClustered + 2:
        return launch_cl<12, 2048, 2>(c, a, grid, sms, s);
    default:
        return launch_cl<8, 2048, 3>(c, a, grid, sms, s);
    }
}

cudaError_t
prepare_sweep_cl()
{
    cudaError_t e = prepare_cl<8, 2048, 2>();
    if (e == cudaSuccess)
        e = prepare_cl<8, 2048, 3>();
    if (e == cudaSuccess)
        e = prepare_cl<12, 2048, 2>();
    return e;
}

}  // namespace fast
}  // namespace aqua
