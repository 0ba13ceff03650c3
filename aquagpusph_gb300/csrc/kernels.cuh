// Kernel-side helpers and launcher declarations shared by the .cu files.
#pragma once

#include "aqua_internal.cuh"

namespace aqua {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;   // keys per block
// sweep variants: threads per block x queued neighbours per thread (the
// staging depth) x queue entry x candidate staging: 0 = (128, 128, 16-bit,
// loads), 1 = (64, 128, 16-bit, loads), 2 = (64, 64, 32-bit, loads),
// 3 = (64, 128, 16-bit, bulk copies), 4 = (64, 64, 32-bit, bulk copies);
// direct sweep (no queue, each candidate group summed as it is loaded):
// 5 = 64 threads, 6 = 128 threads, and with the next group's records
// prefetched by asynchronous copies: 7 = 64 threads, 8 = 128 threads;
// those with the register budget of 28 resident warps per SM (9 = 64,
// 10 = 128 threads), 32 (11, 12) or 36 (13, 14)
// the clustered sweep of the fast 3-D build (BIe walls, midpoint scheme):
// 15 = 8 warps per block for 2 blocks per SM, 16 = 8 warps for 3 blocks,
// 17 = 12 warps for 2 blocks; each stages 2,048 neighbour records per pass
constexpr int kSweepClustered = 15;
constexpr int kSweepVariants = 18;
constexpr int kSweepClusteredDefault = 16;
constexpr unsigned kSweepClusteredBlocks = 3;
inline int
sweep_variant_threads(int v)
{
    if (v >= kSweepClustered)
        return v == kSweepClustered + 2 ? 384 : 256;
    return (v == 0 || (v >= 6 && v % 2 == 0)) ? 128 : 64;
}

// Wendland C2 (Wendland{2D,3D}.hcl:44-66): the constant factors of W and F;
// float products folded at compile time, as the OpenCL compiler folds them
template<int D>
struct WendlandC;
template<>
struct WendlandC<3>
{
    static constexpr float W = 0.08203125f * 0.318309886f;
    static constexpr float F = 0.8203125f * 0.318309886f;
};
template<>
struct WendlandC<2>
{
    static constexpr float W = 0.109375f * 0.318309886f;
    static constexpr float F = 1.09375f * 0.318309886f;
};

// The reference's vec type: float4 in 3-D, float2 in 2-D
template<int D>
struct Vec;
template<>
struct Vec<3>
{
    static constexpr int VS = 4;
    __device__ __forceinline__ static void load(const float* p, uint32_t i, float x[4])
    {
        const float4 v = reinterpret_cast<const float4*>(p)[i];
        x[0] = v.x;
        x[1] = v.y;
        x[2] = v.z;
        x[3] = v.w;
    }
    __device__ __forceinline__ static void store(float* p, uint32_t i, const float x[4])
    {
        reinterpret_cast<float4*>(p)[i] = make_float4(x[0], x[1], x[2], x[3]);
    }
};
template<>
struct Vec<2>
{
    static constexpr int VS = 2;
    __device__ __forceinline__ static void load(const float* p, uint32_t i, float x[4])
    {
        const float2 v = reinterpret_cast<const float2*>(p)[i];
        x[0] = v.x;
        x[1] = v.y;
        x[2] = 0.f;
        x[3] = 0.f;
    }
    __device__ __forceinline__ static void store(float* p, uint32_t i, const float x[4])
    {
        reinterpret_cast<float2*>(p)[i] = make_float2(x[0], x[1]);
    }
};

// link-list / sort launchers (linklist.cu).  `cid` (case of each particle)
// may be NULL: every particle then belongs to case 0.
cudaError_t launch_begin(DevScalars* sc, CaseScalars* cs, uint32_t n_cases,
                         uint2* cells, uint2* wall_range, uint8_t* cell_mark,
                         uint32_t ncap, uint32_t N, cudaStream_t s);
template<int D>
cudaError_t launch_minmax(const Consts& c, const float* r, const int32_t* imove,
                          const uint32_t* cid, uint32_t N, CaseScalars* cs,
                          DevScalars* sc, cudaStream_t s);
template<int D>
cudaError_t launch_ncells(const Consts& c, CaseScalars* cs, uint32_t n_cases,
                          DevScalars* sc, uint32_t ncap, cudaStream_t s);
// icell keys of the positions and the digit histograms (resets the sort
// scratch first); then launch_radix_passes(..., hist_ready = true)
template<int D>
cudaError_t launch_icell_hist(const Consts& c, const float* r,
                              const int32_t* imove, const uint32_t* cid,
                              uint32_t N, const CaseScalars* cs, DevScalars* sc,
                              uint32_t* keys, uint32_t* scratch,
                              uint32_t passes, cudaStream_t s);
cudaError_t launch_radix_passes(uint32_t* keys[2], uint32_t* vals[2],
                                uint32_t n, uint32_t passes, uint32_t* scratch,
                                bool hist_ready, DevScalars* sc,
                                cudaStream_t s);
size_t sort_scratch_words(uint32_t n);
cudaError_t launch_inverse_perm(const uint32_t* perm, uint32_t* inv,
                                uint32_t n, const DevScalars* sc,
                                cudaStream_t s);
cudaError_t launch_ihoc(const uint32_t* keys, uint32_t n, uint32_t* ihoc,
                        uint32_t ncap, const DevScalars* sc, cudaStream_t s);
cudaError_t launch_iota(uint32_t* p, uint32_t n, cudaStream_t s);
uint32_t sort_blocks(uint32_t n);
uint32_t sort_passes(uint32_t key_bits);

// step launchers (step.cu)
struct StepArgs
{
    uint32_t N;
    uint32_t ncap;
    VarSet src;        // previous step's Variables (previous order)
    VarSet dst;        // this step's Variables (new order)
    StepBufs b;
    const uint32_t* skeys;  // sorted cell keys
    const uint32_t* perm;   // sorted -> previous index
    DevScalars* sc;
    CaseScalars* cs;        // per-case scalars (n_cases)
    const CaseMotion* cm;   // per-case prescribed motion (n_cases)
    uint32_t n_cases;
    int extras;        // write the intermediate operators
    int clustered;     // the gather writes rec0/rec1 and the cell list for
                       // the clustered sweep instead of posq/velq/pmq
};
// gather / sweep of the step in the exact (IEEE, no FMA) or fast
// (-use_fast_math) compilation
template<int D>
cudaError_t launch_gather(bool fast, const Consts& c, const StepArgs& a,
                          cudaStream_t s);
template<int D>
cudaError_t launch_sweep(bool fast, const Consts& c, const StepArgs& a,
                         unsigned grid, int variant, cudaStream_t s);
cudaError_t launch_finalize(DevScalars* sc, CaseScalars* cs,
                            const CaseMotion* cm, uint32_t n_cases,
                            cudaStream_t s);
template<int D>
cudaError_t launch_motion(const StepArgs& a, cudaStream_t s);
cudaError_t launch_set_case_ids(uint32_t* cid, const uint32_t* offsets,
                                uint32_t n_cases, uint32_t N, cudaStream_t s);
cudaError_t launch_export_ihoc(const uint2* cells, uint32_t* ihoc,
                               uint32_t ncap, const DevScalars* sc,
                               cudaStream_t s);

// output.cu: report values in original particle order, free-surface sensors
constexpr uint32_t kMaxFsSensors = 64;
constexpr uint32_t kReportValues = AQUA_REPORT_MAX_VALUES;  // report staging
struct FreeSurfaceSensors
{
    float xy[kMaxFsSensors][2];
};
cudaError_t launch_unsorted(const uint32_t* id, const float* src, uint32_t nc,
                            uint32_t N, uint32_t first, uint32_t n, float* out,
                            cudaStream_t s);
cudaError_t launch_unsorted_int(const uint32_t* id, const int32_t* src,
                                uint32_t N, uint32_t first, uint32_t n,
                                float* out, cudaStream_t s);
cudaError_t launch_free_surface(int dims, const float* r, const int32_t* imove,
                                const uint32_t* cid, int32_t case_index,
                                uint32_t N, const FreeSurfaceSensors& sensors,
                                uint32_t n_sensors, float dr, int* keys,
                                float* out, cudaStream_t s);

template<int D>
cudaError_t launch_bi_walls(bool fast, const Consts& c, const StepArgs& a,
                            cudaStream_t s);

namespace exact {
template<int D>
cudaError_t launch_bi_walls_impl(const Consts& c, const StepArgs& a, cudaStream_t s);
template<int D>
cudaError_t launch_gather_impl(const Consts& c, const StepArgs& a, cudaStream_t s);
template<int D>
cudaError_t launch_sweep_impl(const Consts& c, const StepArgs& a, unsigned grid,
                              int variant, cudaStream_t s);
}  // namespace exact
namespace fast {
// clustered sweep: the cluster list then the sweep (variant >= kSweepClustered)
cudaError_t launch_sweep_cl(const Consts& c, const StepArgs& a, unsigned grid,
                            int variant, unsigned sms, cudaStream_t s);
// sets the kernels' dynamic shared memory limit (once, before any capture)
cudaError_t prepare_sweep_cl();
template<int D>
cudaError_t launch_bi_walls_impl(const Consts& c, const StepArgs& a, cudaStream_t s);
template<int D>
cudaError_t launch_gather_impl(const Consts& c, const StepArgs& a, cudaStream_t s);
template<int D>
cudaError_t launch_sweep_impl(const Consts& c, const StepArgs& a, unsigned grid,
                              int variant, cudaStream_t s);
}  // namespace fast

}  // namespace aqua
