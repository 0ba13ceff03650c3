// Output-side kernels: the values a report prints and the free-surface
// elevation sensors, read from the resident (sorted) state.
//
//  - k_unsorted: CalcServer::getUnsortedMem (used by the particle reports,
//    CalcServer/Reports/SetTabFile.cpp:282-287) -- the values of the
//    particles whose original index lies in [first, first + n), in original
//    order.  The state is kept sorted by cell; `id` holds each particle's
//    original index, so one pass over the particles scatters the wanted ones.
//  - k_free_surface: the wave-height sensors of the 3-D dam-break example
//    (examples/3D/spheric_testcase2_dambreak/src/templates/h_sensor.cl:37-61
//    and the "H1".."H4" max reductions of Sensors.xml:43-62): per sensor,
//    h_i = r_i[up] + dr/2 for fluid particles within 2 dr of the sensor along
//    the horizontal axes, 0 for every other particle, and H = max_i h_i
//    (reduction identity -INFINITY).
#include "aqua_internal.cuh"
#include "kernels.cuh"

namespace aqua {

namespace {

__device__ __forceinline__ int
ordered_key(float f)
{
    // monotone map of floats onto signed ints (for integer atomicMax)
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}

__global__ void
k_unsorted(const uint32_t* __restrict__ id, const float* __restrict__ src,
           uint32_t nc, uint32_t N, uint32_t first, uint32_t n,
           float* __restrict__ out)
{
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < N;
         s += gridDim.x * blockDim.x) {
        const uint32_t o = id[s] - first;  // wraps for id < first
        if (o < n)
            for (uint32_t k = 0; k < nc; k++)
                out[(size_t)o * nc + k] = src[(size_t)s * nc + k];
    }
}

__global__ void
k_unsorted_int(const uint32_t* __restrict__ id, const int32_t* __restrict__ src,
               uint32_t N, uint32_t first, uint32_t n, float* __restrict__ out)
{
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < N;
         s += gridDim.x * blockDim.x) {
        const uint32_t o = id[s] - first;
        if (o < n)
            out[o] = __int_as_float(src[s]);
    }
}

__global__ void
k_fs_init(int* keys, uint32_t n)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n)
        keys[k] = ordered_key(-INFINITY);
}

// blockIdx.y = sensor; sensors.xy[s] = its horizontal coordinates (x only in
// 2-D, where the vertical axis is y)
template<int D>
__global__ void
k_free_surface(const float* __restrict__ r, const int32_t* __restrict__ imove,
               const uint32_t* __restrict__ cid, int32_t case_index, uint32_t N,
               FreeSurfaceSensors sensors, float dr, int* keys)
{
    constexpr int VS = D == 3 ? 4 : 2;
    const uint32_t s = blockIdx.y;
    const float sx = sensors.xy[s][0];
    const float sy = sensors.xy[s][1];
    float best = -INFINITY;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N;
         i += gridDim.x * blockDim.x) {
        if (case_index >= 0 && cid[i] != (uint32_t)case_index)
            continue;
        float h = 0.f;
        if (imove[i] > 0) {
            // the sensor's test as written: far = |x| > 2 dr (or |y|)
            const float x = r[(size_t)i * VS] - sx;
            bool near = !(fabsf(x) > 2.f * dr);
            if (D == 3) {
                const float y = r[(size_t)i * VS + 1] - sy;
                near = near && !(fabsf(y) > 2.f * dr);
            }
            if (near)
                h = r[(size_t)i * VS + (D - 1)] + 0.5f * dr;
        }
        best = fmaxf(best, h);
    }
    for (int o = 16; o > 0; o >>= 1)
        best = fmaxf(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0 && best > -INFINITY)
        atomicMax(&keys[s], ordered_key(best));
}

__global__ void
k_fs_decode(const int* keys, uint32_t n, float* out)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) {
        const int i = keys[k];
        out[k] = __int_as_float(i >= 0 ? i : i ^ 0x7fffffff);
    }
}

unsigned
grid_for(uint32_t N, unsigned cap)
{
    const unsigned g = (N + 255) / 256;
    return g == 0 ? 1u : (g < cap ? g : cap);
}

} // namespace

cudaError_t
launch_unsorted(const uint32_t* id, const float* src, uint32_t nc, uint32_t N,
                uint32_t first, uint32_t n, float* out, cudaStream_t s)
{
    k_unsorted<<<grid_for(N, 4096), 256, 0, s>>>(id, src, nc, N, first, n, out);
    return cudaGetLastError();
}

cudaError_t
launch_unsorted_int(const uint32_t* id, const int32_t* src, uint32_t N,
                    uint32_t first, uint32_t n, float* out, cudaStream_t s)
{
    k_unsorted_int<<<grid_for(N, 4096), 256, 0, s>>>(id, src, N, first, n, out);
    return cudaGetLastError();
}

cudaError_t
launch_free_surface(int dims, const float* r, const int32_t* imove,
                    const uint32_t* cid, int32_t case_index, uint32_t N,
                    const FreeSurfaceSensors& sensors, uint32_t n_sensors,
                    float dr, int* keys, float* out, cudaStream_t s)
{
    k_fs_init<<<(n_sensors + 255) / 256, 256, 0, s>>>(keys, n_sensors);
    const dim3 grid(grid_for(N, 1024), n_sensors);
    if (dims == 3)
        k_free_surface<3><<<grid, 256, 0, s>>>(r, imove, cid, case_index, N,
                                               sensors, dr, keys);
    else
        k_free_surface<2><<<grid, 256, 0, s>>>(r, imove, cid, case_index, N,
                                               sensors, dr, keys);
    k_fs_decode<<<(n_sensors + 255) / 256, 256, 0, s>>>(keys, n_sensors, out);
    return cudaGetLastError();
}

}  // namespace aqua
