// Kernel templates of one canonical WCSPH step: the sorted gather and the
// fused neighbour sweep.  This file is compiled twice, into the namespaces
// aqua::exact (step.cu: -fmad=false, IEEE division and square root -- the
// reference's arithmetic, bit-exact with the CPU oracle) and aqua::fast
// (step_fast.cu: -use_fast_math -- FMA contraction and approximate
// division/square root, within the 1e-5 relative tolerance of the
// reference's rates).
//
// The reference runs ~20 kernels and copies per step (basic.xml:132-171 and
// the midpoint/domain/cfd/deltaSPH/BIe/variableTimeStep presets).  Here:
//
//   k_gather  = predictor backups + Domain + sort stage1/stage2 + EOS +
//               Binormal + midpoint init copies + midpoint advance +
//               midpoint EOS (one pass over the sorted order; it also writes
//               the cell table and packs the neighbour data)
//   k_sweep   = cfd Shepard + cfd interactions + cfd sensors + sensors
//               renormalization + cfd lap p + BIe interactions, in ONE
//               traversal of the 3^D neighbour cells, then per particle:
//               BIe rates + cfd rates + delta-SPH + BIe elastic bounce +
//               midpoint relax + corrector + BIe pst + variable time step
//               + block min of dt_var (grid minimum by atomicMin)
//
// With the improved Euler scheme (basic/time_scheme/improved_euler.xml, BI
// walls) k_gather runs the improved_euler.cl predictor in place of the
// midpoint backups, copies and advance, and the sweep epilogue its corrector
// in place of the midpoint relax and corrector.
//
// Every accumulator visits its neighbours in the reference order (27 cells,
// x offset outermost; particles of a cell in sorted order) and each
// expression keeps the reference's evaluation order.
//
// Work distribution of the sweep: a warp takes a chunk of <= 32 particles
// of ONE cell (chunks are built by k_chunks, fetched dynamically), so all
// lanes walk the same 27 neighbour cells and every neighbour load is a
// warp-wide broadcast.
//
// Reference kernels (resources/Scripts/...): basic/time_scheme/midpoint.cl,
// basic/time_scheme/improved_euler.cl,
// basic/Domain.cl, basic/Sort.cl, basic/EOS.cl, basic/Binormal.cl,
// basic/Shepard.cl, cfd/Interactions.cl, cfd/Sensors.cl,
// cfd/SensorsRenormalization.cl, basic/deltaSPH.cl (lapp, deltaSPH),
// cfd/Boundary/BIe/{Interactions,Rates,ElasticBounce,PST}.cl, cfd/Rates.cl,
// cfd/TimeStep.cl, KernelFunctions/Wendland{2D,3D}.hcl.
//
// This header has no include guard: it is meant to be included once per
// namespace by step.cu and step_fast.cu.

namespace {

constexpr uint32_t kBulkWaitLimit = 1u << 20;  // bounded mbarrier polls

// The fast build (step_fast.cu) factors the fluid pair sums of the direct
// sweep (reassociated, within the fast build's tolerance); the exact build
// keeps the reference's expressions
constexpr bool kFastArith = AQUA_FAST_ARITH != 0;

// How the sweep hands in-support candidates to the pair arithmetic: per-lane
// ring queues drained with full warps, or directly, each survivor of a group
// summed at once by the lanes it reaches
constexpr int kSweepQueue = 0;
constexpr int kSweepDirect = 1;

// Ampere-style asynchronous copies global -> shared (no registers held while
// in flight), grouped and waited for per thread
__device__ __forceinline__ void
cp_async_16(void* smem, const void* gmem)
{
    const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n"
                 :: "r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void
cp_async_8(void* smem, const void* gmem)
{
    const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n"
                 :: "r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void
cp_async_commit()
{
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}
// waits until at most one committed group of this thread is in flight
__device__ __forceinline__ void
cp_async_wait_all_but_one()
{
    asm volatile("cp.async.wait_group 1;\n" ::: "memory");
}

// Wendland C2 kernel (Wendland{2D,3D}.hcl:44-66); constants in WendlandC
// (kernels.cuh)
template<int D>
__device__ __forceinline__ float
kernel_w(float q)
{
    const float a = 2.f - q;
    float w = WendlandC<D>::W * (1.f + 2.f * q);
    w = w * a;
    w = w * a;
    w = w * a;
    return w * a;
}

template<int D>
__device__ __forceinline__ float
kernel_f(float q)
{
    const float a = 2.f - q;
    float f = WendlandC<D>::F * a;
    f = f * a;
    return f * a;
}

// Boundary-integral Shepard factor (KernelFunctions/Wendland{2D,3D}.hcl:
// kernelS_P, the polynomial part, and kernelS_D, the analytic part)
template<int D>
__device__ __forceinline__ float
kernel_sp(float q)
{
    const float q2 = q * q;
    const float q3 = q2 * q;
    if (D == 3) {
        constexpr float wcon = 0.08203125f * 0.318309886f;
        return wcon * (0.25f * q3 * q2 - 2.142857f * q2 * q2 + 6.666667f * q3 -
                       8.f * q2 + 5.333333f);
    } else {
        constexpr float wcon = 0.109375f * 0.318309886f;
        return wcon * (0.285714f * q3 * q2 - 2.5f * q2 * q2 + 8.f * q3 -
                       10.f * q2 + 8.f);
    }
}

__device__ __forceinline__ float
acospi_f(float x)
{
    return acosf(x) / 3.14159265f;
}

__device__ __forceinline__ float
omega_f(float a, float b)
{
    const float a2 = a * a;
    const float b2 = b * b;
    const float v = sqrtf((1.f + a2 + b2) / ((1.f + a2) * (1.f + b2)));
    return acospi_f((1.f < v) ? 1.f : v);
}

__device__ __forceinline__ float
sign_f(float x)
{
    return (x > 0.f) ? 1.f : ((x < 0.f) ? -1.f : 0.f);
}

template<int D>
__device__ __forceinline__ float
kernel_sd(float d, float t, float b, float s)
{
    if (D == 3) {
        const float wcon = 0.25f;
        const float dr = 0.5f * sqrtf(s);
        const float t1 = (t - dr) / d, t2 = (t + dr) / d;
        const float b1 = (b - dr) / d, b2 = (b + dr) / d;
        const float st = sign_f(t1), sb = sign_f(b1);
        return -wcon * (omega_f(t2, b2) - st * omega_f(t1, b2) -
                        sb * omega_f(t2, b1) + st * sb * omega_f(t1, b1));
    } else {
        constexpr float wcon = 0.5f * 0.318309886f;
        const float dr = 0.5f * s;
        return -wcon * (atanf((t + dr) / d) - atanf((t - dr) / d));
    }
}

__device__ __forceinline__ float
cl_min(float x, float y)
{
    return (y < x) ? y : x;
}
__device__ __forceinline__ float
cl_max(float x, float y)
{
    return (x < y) ? y : x;
}

template<int D>
__device__ __forceinline__ float
dot_d(const float* a, const float* b)
{
    float s = a[0] * b[0];
    s = s + a[1] * b[1];
    if (D == 3)
        s = s + a[2] * b[2];
    return s;
}

// dot over the storage vector (float4 in 3-D, including w)
template<int D>
__device__ __forceinline__ float
dot_full(const float* a, const float* b)
{
    float s = a[0] * b[0];
    s = s + a[1] * b[1];
    if (D == 3) {
        s = s + a[2] * b[2];
        s = s + a[3] * b[3];
    }
    return s;
}

// Neighbour cell k (0 .. 3^D-1) of cell c in the reference order: x offset
// outermost, then y, then z
template<int D>
__device__ __forceinline__ uint32_t
neighbour_cell(uint32_t c, int k, uint32_t nx, uint32_t nxy)
{
    if (D == 3) {
        const int ci = k / 9 - 1, cj = (k / 3) % 3 - 1, ck = k % 3 - 1;
        return c + (uint32_t)ci + (uint32_t)cj * nx + (uint32_t)ck * nxy;
    } else {
        const int ci = k / 3 - 1, cj = k % 3 - 1;
        return c + (uint32_t)ci + (uint32_t)cj * nx;
    }
}

template<int D>
__device__ __forceinline__ void
load_normal(const float* normal, uint32_t j, float n[3])
{
    if (D == 3) {
        const float4 v = reinterpret_cast<const float4*>(normal)[j];
        n[0] = v.x;
        n[1] = v.y;
        n[2] = v.z;
    } else {
        const float2 v = reinterpret_cast<const float2*>(normal)[j];
        n[0] = v.x;
        n[1] = v.y;
        n[2] = 0.f;
    }
}

}  // namespace

// ------------------------------------------------------------------ gather

template<int D>
__global__ void __launch_bounds__(256)
k_gather(Consts c, StepArgs a)
{
    constexpr int VS = Vec<D>::VS;
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.N || a.sc->err)
        return;
    const uint32_t N = a.N;
    const uint32_t key = a.skeys[s];
    if (key >= a.ncap) {
        atomicOr(&a.sc->err, kErrCapacity);
        return;
    }
    const uint32_t o = a.perm[s];
    a.b.id_sorted[o] = s;
    if (s == 0 || a.skeys[s - 1] != key)
        a.b.cells[key].x = s;
    if (s == N - 1 || a.skeys[s + 1] != key)
        a.b.cells[key].y = s + 1;

    const VarSet& S = a.src;
    const VarSet& T = a.dst;
    const uint32_t kc = S.cid[o];
    const float dt = a.cs[kc].dt;
    const float hdt = 0.5f * dt;
    T.cid[s] = kc;

    const bool heun = c.scheme == AQUA_SCHEME_IMPROVED_EULER;
    int im = S.imove[o];
    float r[4] = { 0.f, 0.f, 0.f, 0.f };
    Vec<D>::load(S.r, o, r);
    float u0[4] = { 0.f, 0.f, 0.f, 0.f }, ain[4] = { 0.f, 0.f, 0.f, 0.f };
    Vec<D>::load(S.u, o, u0);
    Vec<D>::load(S.dudt, o, ain);
    float rho_in = S.rho[o];
    const float drhodt_in = S.drhodt[o];
    if (heun) {
        // improved_euler.cl predictor: an explicit second-order Taylor step
        // from the last state (DT = 0 for imove <= 0), before Domain
        const float DT = (im <= 0) ? 0.f : dt;
        const float DT2 = 0.5f * DT * DT;
        for (int k = 0; k < VS; k++) {
            r[k] = r[k] + DT * u0[k] + DT2 * ain[k];
            u0[k] = u0[k] + DT * ain[k];
        }
        rho_in = rho_in + DT * drhodt_in;
    }

    // Domain (on the predictor output) + sort stage1
    bool removed = false;
    if (im > -255) {
        bool out = false;
        for (int k = 0; k < D; k++)
            out = out || isnan(r[k]) || isinf(r[k]) || r[k] < c.domain_min[k] ||
                  r[k] > c.domain_max[k];
        if (out) {
            removed = true;
            im = -256;
            for (int k = 0; k < VS; k++)
                r[k] = c.domain_max[k];
        }
    }
    const uint32_t set_raw = S.iset[o];
    // out-of-range sets read set 0 (the per-set arrays hold n_sets entries)
    const uint32_t set = set_raw < c.n_sets ? set_raw : 0u;
    T.id[s] = S.id[o];
    T.iset[s] = set_raw;
    T.imove[s] = im;
    float nrm[4], tng[4], bn[4] = { 0.f, 0.f, 0.f, 0.f };
    Vec<D>::load(S.normal, o, nrm);
    Vec<D>::load(S.tangent, o, tng);
    // Binormal.cl
    if (D == 3) {
        bn[0] = nrm[1] * tng[2] - nrm[2] * tng[1];
        bn[1] = nrm[2] * tng[0] - nrm[0] * tng[2];
        bn[2] = nrm[0] * tng[1] - nrm[1] * tng[0];
        bn[3] = 0.f;
    } else {
        tng[0] = nrm[1];
        tng[1] = -nrm[0];
    }
    Vec<D>::store(T.normal, s, nrm);
    Vec<D>::store(T.tangent, s, tng);
    Vec<D>::store(T.binormal, s, bn);

    // sort stage2 (+ Domain zeroing of u_in and m)
    const float m = removed ? 0.f : S.m[o];
    float uin[4] = { 0.f, 0.f, 0.f, 0.f };
    if (!removed)
        for (int k = 0; k < 4; k++)
            uin[k] = u0[k];

    // midpoint advance (imove > 0), midpoint EOS; improved Euler: the EOS of
    // the sorted predictor output
    float uh[4];
    float rho_h = rho_in;
    for (int k = 0; k < 4; k++)
        uh[k] = uin[k];
    if (!heun && im > 0) {
        for (int k = 0; k < VS; k++)
            uh[k] = uin[k] + hdt * ain[k];
        rho_h = rho_in + hdt * drhodt_in;
    }
    float p;
    if (im > 0 || im == -1)
        p = c.p0 + c.cs * c.cs * (rho_h - c.refd[set]);
    else
        p = S.p[s];  // the pressure Variable is not permuted by the sort

    // The clustered sweep (fast 3-D build, midpoint scheme, every cell
    // swept) writes r, u, dudt, drhodt and rho of every fluid particle and
    // reads none of them before: the gather leaves them out there.
    const bool swept = a.clustered && !c.sample_on && !heun && im == 1;
    if (!swept) {
        Vec<D>::store(T.r, s, r);
        Vec<D>::store(T.u, s, uh);
    }
    Vec<D>::store(a.b.r_in, s, r);
    Vec<D>::store(a.b.u_in, s, uin);
    Vec<D>::store(a.b.dudt_in, s, ain);
    a.b.drhodt_in[s] = drhodt_in;
    if (swept) {
    } else if (heun) {
        // Without the midpoint init copies nothing permutes the rates
        // Variables: until the rates are computed (fluid only, cfd/Rates.cl)
        // dudt and drhodt keep the last step's order, and BI/GradP.cl reads
        // a wall's dudt at its new sorted index from them.
        float a_old[4] = { 0.f, 0.f, 0.f, 0.f };
        Vec<D>::load(S.dudt, s, a_old);
        Vec<D>::store(T.dudt, s, a_old);
        T.drhodt[s] = S.drhodt[s];
    } else {
        Vec<D>::store(T.dudt, s, ain);
        T.drhodt[s] = drhodt_in;
    }
    if (!swept)
        T.rho[s] = rho_h;
    a.b.rho_in[s] = rho_in;
    T.m[s] = m;
    T.p[s] = p;
    if (a.clustered) {
        // neighbour records of the clustered sweep: fluid (volume m/rho
        // times the kernel's CONW W-factor, velocity, pressure), boundary
        // element (-area, normal, u.normal), anything else (0: no neighbour
        // sums)
        float w0 = 0.f;
        float4 r1 = make_float4(uh[0], uh[1], D == 3 ? uh[2] : 0.f, p);
        if (im == 1) {
            w0 = c.w_conw * (m / rho_h);  // CONW W-factor * volume
        } else if (im == -3) {
            w0 = -m;
            float un = uh[0] * nrm[0] + uh[1] * nrm[1];
            if (D == 3)
                un = un + uh[2] * nrm[2];
            r1 = make_float4(nrm[0], nrm[1], D == 3 ? nrm[2] : 0.f, un);
        }
        a.b.rec0[s] = make_float4(r[0], r[1], D == 3 ? r[2] : 0.f, w0);
        a.b.rec1[s] = r1;
    } else {
        a.b.posq[s] = make_float4(r[0], r[1], D == 3 ? r[2] : 0.f, __int_as_float(im));
        a.b.velq[s] = make_float4(uh[0], uh[1], D == 3 ? uh[2] : 0.f, rho_h);
        a.b.pmq[s] = make_float2(p, m);
    }
    if (im == -3) {
        // the cell's boundary elements lie within [x, y) of its particles
        atomicMin(&a.b.wall_range[key].x, s);
        atomicMax(&a.b.wall_range[key].y, s + 1);
    }
    if (c.sample_on && im == 0) {
        // rate sample: the cells around a probe are always swept
        const uint32_t nx = a.cs[kc].n_cells[0];
        const uint32_t nxy = nx * a.cs[kc].n_cells[1];
        for (int k = 0; k < ((D == 3) ? 27 : 9); k++)
            a.b.cell_mark[neighbour_cell<D>(key, k, nx, nxy)] = 1;
    }
}

// ------------------------------------------------------------------- sweep

// Everything the sweep does for sorted particle i; returns its dt_var (or
// +inf when the particle has none).  All 32 lanes of a warp call it for
// particles of the same cell (`valid` is false for the lanes past the end of
// the chunk), so the neighbour scan below is warp-uniform.
//
// The neighbour loop runs in two phases so that the expensive pair
// arithmetic executes with full warps: the scan walks the candidates of the
// 3^D cells in the reference order and appends the ones inside the support
// to this lane's ring queue in shared memory (one column per thread); the
// drain pops the queue in order and accumulates.  Every sum keeps the
// reference's order.  A queue entry (QE) is either the neighbour's sorted
// index (32 bits) or, to halve the queue's shared memory, 16 bits: the
// neighbour-cell slot k (5 bits) and the candidate's offset in that cell
// (11 bits), resolved through `cstart`, the first sorted index of the 3^D
// neighbour cells of the warp's cell.  The scan checks the queues every 32
// candidates, where they have room for at least 32 more, so a queue never
// overflows.
template<int D, int NT, int NQ, typename QE, bool BULK, bool BI, int MODE>
__device__ __forceinline__ float
sweep_particle(const Consts& c, const StepArgs& a, uint32_t i, bool valid,
               QE* queue, uint32_t* cstart, float4* grp2, uint64_t* mbar,
               uint32_t& phases, float4* vel_s, float2* pm_s, float* box_s)
{
    constexpr int VS = Vec<D>::VS;
    constexpr int NC = (D == 3) ? 27 : 9;
    const VarSet& T = a.dst;
    const CaseScalars& cas = a.cs[T.cid[i]];
    const float dt = cas.dt;
    const float hdt = 0.5f * dt;
    const float4 pi = a.b.posq[i];
    const int im = __float_as_int(pi.w);
    const uint32_t nx = cas.n_cells[0];
    const uint32_t nxy = cas.n_cells[0] * cas.n_cells[1];
    const uint32_t key_i = a.skeys[i];
    const bool fluid = valid && (im == 1), sensor = valid && (im == 0);
    // BIe: the Shepard sum runs for -3 <= imove <= 1 (cfd/Shepard.cl); BI:
    // the walls are handled by k_bi_walls, fluid and probes take fluid
    // neighbours only here and the walls in the epilogue
    constexpr bool bie = !BI;  // the wall formulation is a compile-time choice
    const bool want_shep = valid && (bie ? (im >= -3) && (im <= 1)
                                         : (im == 0) || (im == 1));

    float shep = 0.f;
    float gp[3] = { 0.f, 0.f, 0.f }, lu[3] = { 0.f, 0.f, 0.f };
    float gw[3] = { 0.f, 0.f, 0.f };
    float du = 0.f, lp = 0.f, dbi = 0.f;
    // a probe takes no fluid sums: its interpolated velocity, density and
    // pressure (cfd/Sensors.cl) accumulate in gp, du and lp
    const float4 vi = a.b.velq[i];
    const float rho_i = vi.w;
    const float p_i = a.b.pmq[i].x;
    const float ri[3] = { pi.x, pi.y, pi.z };
    const float uiv[3] = { vi.x, vi.y, vi.z };

    // One neighbour j of the sums (its packed records pj, vj, pmj), taken in
    // visiting order; the support test is the reference's q >= SUPPORT.
    auto pair = [&](uint32_t j, const float4 pj, const float4 vj,
                    const float2 pmj) {
        const int jm = __float_as_int(pj.w);
        float d[3];
        d[0] = pj.x - ri[0];
        d[1] = pj.y - ri[1];
        d[2] = (D == 3) ? pj.z - ri[2] : 0.f;
        const float rr = dot_d<D>(d, d);
        const float q = sqrtf(rr) / c.H;
        if (q >= c.SUPPORT)
            return;
        if (jm == 1) {
            const float rho_j = vj.w, m_j = pmj.y;
            const float wj = kernel_w<D>(q) * c.CONW * m_j / rho_j;
            shep = shep + wj;
            if (j == i)
                return;
            if (fluid) {
                const float p_j = pmj.x;
                float dv[3];
                dv[0] = vj.x - uiv[0];
                dv[1] = vj.y - uiv[1];
                dv[2] = (D == 3) ? vj.z - uiv[2] : 0.f;
                const float udr = dot_d<D>(dv, d);
                const float f_ij = kernel_f<D>(q) * c.CONF * m_j;
                const float rr_ij = rho_i * rho_j;
                const float sgp = (p_i + p_j) / rr_ij * f_ij;
                const float slu = f_ij * 2.f / rr_ij;
                for (int kk = 0; kk < D; kk++) {
                    gp[kk] = gp[kk] + sgp * d[kk];
                    lu[kk] = lu[kk] + slu * dv[kk];
                }
                du = du + udr * f_ij * rho_i / rho_j;
                lp = lp + (p_j - p_i) * (f_ij / rho_j);
            } else if (sensor) {
                gp[0] = gp[0] + vj.x * wj;
                gp[1] = gp[1] + vj.y * wj;
                if (D == 3)
                    gp[2] = gp[2] + vj.z * wj;
                du = du + rho_j * wj;
                lp = lp + pmj.x * wj;
            }
        } else {
            // boundary element: BIe wall sums (fluid i only)
            float nj[3];
            load_normal<D>(a.dst.normal, j, nj);
            const float uj[3] = { vj.x, vj.y, vj.z };
            const float wa = kernel_w<D>(q) * c.CONW * pmj.y;
            float g[3];
            for (int kk = 0; kk < D; kk++) {
                g[kk] = nj[kk] * wa;
                gw[kk] = gw[kk] + g[kk];
            }
            dbi = dbi - dot_d<D>(uj, g);
        }
    };

    // Separation r_ij = r_j - r_i and its square (one expression for every
    // path, so the fast build contracts it the same way everywhere)
    auto sep = [&](const float4 pj, float& d0, float& d1, float& d2) -> float {
        d0 = pj.x - ri[0];
        d1 = pj.y - ri[1];
        d2 = (D == 3) ? pj.z - ri[2] : 0.f;
        float rr = d0 * d0 + d1 * d1;
        if (D == 3)
            rr = rr + d2 * d2;
        return rr;
    };
    // The fast build's pair sums: vj.w carries the neighbour's volume
    // m_j/rho_j, CONW and CONF are folded into the kernel factors, and the
    // fluid sums leave out the factors of particle i (1/rho_i, 2/rho_i,
    // rho_i), applied once after the loop.  The self pair adds exact zeros
    // to every sum but Shepard's, so it takes no test.
    auto pair_v = [&](uint32_t j, const float4 pj, const float4 vj,
                      const float2 pmj, float d0, float d1, float d2,
                      float rr) {
        const int jm = __float_as_int(pj.w);
        const float q = sqrtf(rr) * c.inv_H;
        if (q >= c.SUPPORT)
            return;
        const float tq = 2.f - q;
        const float tq2 = tq * tq;
        const float wp = c.w_conw * (1.f + 2.f * q) * tq2 * tq2;  // W(q) CONW
        if (jm == 1) {
            const float wj = wp * vj.w;
            shep = shep + wj;
            if (fluid) {
                const float gf = c.f_conf * tq2 * tq * vj.w;  // F(q) CONF m/rho
                const float dv0 = vj.x - uiv[0], dv1 = vj.y - uiv[1];
                const float dv2 = (D == 3) ? vj.z - uiv[2] : 0.f;
                float udr = dv0 * d0 + dv1 * d1;
                if (D == 3)
                    udr = udr + dv2 * d2;
                const float t = (p_i + pmj.x) * gf;
                gp[0] = gp[0] + t * d0;
                gp[1] = gp[1] + t * d1;
                lu[0] = lu[0] + gf * dv0;
                lu[1] = lu[1] + gf * dv1;
                if (D == 3) {
                    gp[2] = gp[2] + t * d2;
                    lu[2] = lu[2] + gf * dv2;
                }
                du = du + udr * gf;
                lp = lp + (pmj.x - p_i) * gf;
            } else if (sensor) {
                gp[0] = gp[0] + vj.x * wj;
                gp[1] = gp[1] + vj.y * wj;
                if (D == 3)
                    gp[2] = gp[2] + vj.z * wj;
                du = du + wp * pmj.y;  // rho_j W CONW m_j / rho_j
                lp = lp + pmj.x * wj;
            }
        } else {
            // boundary element: BIe wall sums (fluid i only)
            float nj[3];
            load_normal<D>(a.dst.normal, j, nj);
            const float uj[3] = { vj.x, vj.y, vj.z };
            const float wa = wp * pmj.y;
            float g[3];
            for (int kk = 0; kk < D; kk++) {
                g[kk] = nj[kk] * wa;
                gw[kk] = gw[kk] + g[kk];
            }
            dbi = dbi - dot_d<D>(uj, g);
        }
    };

    uint32_t qh = 0, qt = 0;  // ring queue head / tail
    // The drain is software-pipelined: the records of the next queued
    // neighbour are loaded while the current pair is computed.
    auto drain = [&](uint32_t upto) {
        if (qh >= upto)
            return;
        uint32_t jn;
        float4 pn, vn;
        float2 mn;
        auto fetch = [&](uint32_t h) {
            const uint32_t e = queue[(h & (NQ - 1)) * NT];
            if constexpr (sizeof(QE) == 2)
                jn = cstart[e >> 11] + (e & 2047u);
            else
                jn = e;
            pn = a.b.posq[jn];
            vn = a.b.velq[jn];
            mn = a.b.pmq[jn];
        };
        fetch(qh);
        for (; qh < upto; qh++) {
            const uint32_t j = jn;
            const float4 pj = pn;
            const float4 vj = vn;
            const float2 pmj = mn;
            if (qh + 1 < upto)
                fetch(qh + 1);
            if constexpr (kFastArith) {
                float d0, d1, d2;
                const float rr = sep(pj, d0, d1, d2);
                float4 vv = vj;
                vv.w = pmj.y / vj.w;  // the volume m_j / rho_j
                pair_v(j, pj, vv, pmj, d0, d1, d2, rr);
            } else {
                pair(j, pj, vj, pmj);
            }
        }
    };

    // box of the positions of the lanes that take neighbours (empty when
    // none does); candidates farther than the support from it are skipped
    // (warp-uniform: kept in shared memory, read back per group, so that it
    // holds no registers through the candidate loop)
    for (int d = 0; d < 3; d++) {
        float lo = want_shep ? ri[d] : INFINITY;
        float hi = want_shep ? ri[d] : -INFINITY;
        for (int o = 16; o > 0; o >>= 1) {
            lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        }
        if ((threadIdx.x & 31) == 0) {
            box_s[d] = lo;
            box_s[3 + d] = hi;
        }
    }
    __syncwarp();
    const volatile float* box = box_s;
    // a margin over the per-lane bound covers rounding differences between
    // the box distance and the lanes' own distances
    const float q2_box = c.q2_reject * 1.001f;

    const int lane = threadIdx.x & 31;
    if constexpr (sizeof(QE) == 2) {
        // first sorted index of each neighbour cell (same for the whole warp)
        if (lane < NC)
            cstart[lane] = a.b.cells[neighbour_cell<D>(key_i, lane, nx, nxy)].x;
        __syncwarp();
    }
    // The candidates are visited in groups of up to 32 (cell by cell, in the
    // reference order).  With BULK the bulk-copy engine copies each group's
    // packed positions into a shared-memory buffer one group ahead (two
    // buffers per warp, completion tracked by an mbarrier each), so the copy
    // of the next group overlaps the work on the current one; without it
    // the lanes load the group themselves (one coalesced load).
    auto advance = [&](int& kk, uint2& se, uint32_t& g) -> bool {
        g += 32u;
        while (g >= se.y - se.x) {
            if (++kk >= NC)
                return false;
            se = a.b.cells[neighbour_cell<D>(key_i, kk, nx, nxy)];
            g = 0;
            if (sizeof(QE) == 2 && se.y - se.x > 2048u) {
                // the 11-bit offsets cannot address such a cell
                if (lane == 0)
                    atomicOr(&a.sc->err, kErrCapacity);
                se.y = se.x;
            }
        }
        return true;
    };
    auto issue = [&](int b, const uint2 se, uint32_t g) {
        if constexpr (BULK && MODE != kSweepQueue) {
            // every lane copies its candidate's three records; committed by
            // the caller as one group per candidate group
            const uint32_t j = se.x + g + lane;
            if (g + lane < se.y - se.x) {
                cp_async_16(grp2 + 32 * b + lane, a.b.posq + j);
                cp_async_16(vel_s + 32 * b + lane, a.b.velq + j);
                cp_async_8(pm_s + 32 * b + lane, a.b.pmq + j);
            }
        } else if (BULK && lane == 0) {
            const uint32_t bytes = min(32u, se.y - se.x - g) * 16u;
            const uint32_t mb = (uint32_t)__cvta_generic_to_shared(&mbar[b]);
            const uint32_t dst = (uint32_t)__cvta_generic_to_shared(grp2 + 32 * b);
            const uint64_t src = (uint64_t)__cvta_generic_to_global(a.b.posq + se.x + g);
            // earlier generic reads of the buffer before the async write
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n"
                         :: "r"(mb), "r"(bytes) : "memory");
            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
                         "[%0], [%1], %2, [%3];\n"
                         :: "r"(dst), "l"(src), "r"(bytes), "r"(mb) : "memory");
        }
    };
    auto wait = [&](int b) -> bool {
        if constexpr (MODE != kSweepQueue) {
            // the group before the newest is this one
            cp_async_wait_all_but_one();
            __syncwarp();
            return true;
        }
        const uint32_t mb = (uint32_t)__cvta_generic_to_shared(&mbar[b]);
        const uint32_t par = (phases >> b) & 1u;
        uint32_t done = 0;
        for (uint32_t it = 0; it < kBulkWaitLimit && !done; it++)
            asm volatile("{\n.reg .pred p;\n"
                         "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                         "selp.u32 %0, 1, 0, p;\n}\n"
                         : "=r"(done) : "r"(mb), "r"(par) : "memory");
        phases ^= 1u << b;
        // test switch: a wait that completed counts as timed out
        return __all_sync(0xffffffffu, done != 0) && !c.debug_fake_timeout;
    };

    int k = -1;
    uint2 se = make_uint2(0u, 0u);
    uint32_t g = 0xFFFFFFE0u;  // advance() wraps it to the first group
    bool have = advance(k, se, g);
    int buf = 0;
    if (BULK && have)
        issue(0, se, g);
    if (BULK && MODE != kSweepQueue)
        cp_async_commit();
    while (have) {
        int kn = k;
        uint2 sen = se;
        uint32_t gn = g;
        const bool hn = advance(kn, sen, gn);
        if (BULK && hn)
            issue(buf ^ 1, sen, gn);
        if (BULK && MODE != kSweepQueue)
            cp_async_commit();  // possibly empty: one group per iteration
        // warp-uniform checkpoint: make room for the next 32 candidates,
        // first draining the entries every lane has (full warps)
        constexpr uint32_t room = NQ > 32 ? (uint32_t)(NQ - 32) : 0u;
        if (MODE == kSweepQueue && __any_sync(0xffffffffu, qt - qh > room)) {
            const uint32_t fill = qt - qh;
            const uint32_t common = __reduce_min_sync(
                0xffffffffu, want_shep ? fill : 0xffffffffu);
            drain(qh + min(common, fill));
            if (__any_sync(0xffffffffu, qt - qh > room))
                drain(qt);
        }
        const uint32_t count = se.y - se.x;
        const uint32_t gend = min(g + 32u, count);
        float4* grp = grp2 + 32 * buf;
        if constexpr (BULK) {
            if (!wait(buf)) {
                if (lane == 0)
                    atomicOr(&a.sc->err, kErrTimeout);
                if (hn)
                    wait(buf ^ 1);  // the copy in flight, again bounded
                break;
            }
        } else {
            if (g + lane < gend)
                grp[lane] = a.b.posq[se.x + g + lane];
            __syncwarp();
        }
        // lane-parallel pre-filter of the candidates of this group: drop
        // those farther than the support from the box of the chunk's
        // particles (no lane can take them); the survivors are then tested
        // per lane in their visiting order
        bool cand = false;
        if (g + lane < gend) {
            const float4 pc = grp[lane];
            const int jm = __float_as_int(pc.w);
            const float bx = fmaxf(fmaxf(box[0] - pc.x, pc.x - box[3]), 0.f);
            const float by = fmaxf(fmaxf(box[1] - pc.y, pc.y - box[4]), 0.f);
            float bb = bx * bx + by * by;
            if (D == 3) {
                const float bz = fmaxf(fmaxf(box[2] - pc.z, pc.z - box[5]), 0.f);
                bb = bb + bz * bz;
            }
            cand = (jm == 1 || jm == -3) && bb < q2_box;
        }
        uint32_t bal = __ballot_sync(0xffffffffu, cand);
        if constexpr (MODE != kSweepQueue) {
            // the survivors' other records (prefetched with the group, or
            // one coalesced load per lane); then every survivor, in visiting
            // order, is summed at once by the lanes whose particle it reaches
            float4* vel = vel_s + (BULK ? 32 * buf : 0);
            float2* pm = pm_s + (BULK ? 32 * buf : 0);
            if constexpr (!BULK) {
                if (cand) {
                    vel[lane] = a.b.velq[se.x + g + lane];
                    pm[lane] = a.b.pmq[se.x + g + lane];
                }
                __syncwarp();
            }
            if constexpr (kFastArith) {
                // the survivor's volume m_j / rho_j in place of its density
                if (cand)
                    vel[lane].w = pm[lane].y / vel[lane].w;
                __syncwarp();
            }
            while (bal) {
                const uint32_t b = __ffs(bal) - 1;
                bal &= bal - 1;
                const float4 pj = grp[b];
                const int jm = __float_as_int(pj.w);
                float d0, d1, d2;
                const float rr = sep(pj, d0, d1, d2);
                const bool take = want_shep &&
                                  (jm == 1 || (bie && fluid && jm == -3)) &&
                                  rr < c.q2_reject;
                if (take) {
                    if constexpr (kFastArith)
                        pair_v(se.x + g + b, pj, vel[b], pm[b], d0, d1, d2, rr);
                    else
                        pair(se.x + g + b, pj, vel[b], pm[b]);
                }
            }
        }
        auto consider = [&](const float4 pj, uint32_t off) {
            const int jm = __float_as_int(pj.w);
            const float d0 = pj.x - ri[0], d1 = pj.y - ri[1];
            float rr = d0 * d0 + d1 * d1;
            if (D == 3) {
                const float d2 = pj.z - ri[2];
                rr = rr + d2 * d2;
            }
            const bool take = want_shep &&
                              (jm == 1 || (bie && fluid && jm == -3)) &&
                              rr < c.q2_reject;
            if (take) {
                if constexpr (sizeof(QE) == 2)
                    queue[(qt & (NQ - 1)) * NT] = (QE)(((uint32_t)k << 11) | off);
                else
                    queue[(qt & (NQ - 1)) * NT] = se.x + off;
                qt++;
            }
        };
        while (MODE == kSweepQueue && bal) {
            // two survivors per iteration, in visiting order
            const uint32_t b0 = __ffs(bal) - 1;
            bal &= bal - 1;
            const bool two = bal != 0;
            const uint32_t b1 = two ? (uint32_t)(__ffs(bal) - 1) : b0;
            if (two)
                bal &= bal - 1;
            const float4 p0 = grp[b0];
            const float4 p1 = grp[b1];
            consider(p0, g + b0);
            if (two)
                consider(p1, g + b1);
        }
        __syncwarp();  // the buffer is rewritten by the group after next
        k = kn;
        se = sen;
        g = gn;
        have = hn;
        buf ^= 1;
    }
    if constexpr (MODE == kSweepQueue)
        drain(qt);
    if (!valid)
        return INFINITY;
    if constexpr (kFastArith) {
        // the factors of particle i left out of the fluid sums
        if (fluid) {
            const float ir = 1.f / rho_i;
            const float ir2 = 2.f * ir;
            for (int kk = 0; kk < D; kk++) {
                gp[kk] = gp[kk] * ir;
                lu[kk] = lu[kk] * ir2;
            }
            du = du * rho_i;
        }
    }
    if constexpr (BI) {
        // BI walls: the analytic Shepard factor (BI/Shepard.cl compute) of
        // fluid particles and probes, and the wall terms of the fluid
        // particles (BI/Interactions.cl) added onto the completed fluid
        // sums, walls in visiting order
        if (im == -3)
            return c.dt_fixed;  // done by k_bi_walls
        shep = 1.f;
        bool self_added = false;
        for (int k = 0; k < NC; k++) {
            const uint32_t cn = neighbour_cell<D>(key_i, k, nx, nxy);
            const uint2 se = a.b.wall_range[cn];  // empty: x > y
            for (uint32_t j = se.x; j < se.y; j++) {
                const float4 pj = a.b.posq[j];
                if (__float_as_int(pj.w) != -3)
                    continue;
                float d[3];
                d[0] = pj.x - ri[0];
                d[1] = pj.y - ri[1];
                d[2] = (D == 3) ? pj.z - ri[2] : 0.f;
                const float q = sqrtf(dot_d<D>(d, d)) / c.H;
                if (q >= c.SUPPORT)
                    continue;
                float nj[3], tj[3], bj[3];
                load_normal<D>(a.dst.normal, j, nj);
                load_normal<D>(a.dst.tangent, j, tj);
                load_normal<D>(a.dst.binormal, j, bj);
                const float area = a.b.pmq[j].y;
                const float rn = dot_d<D>(d, nj);
                if ((rn > -1e-8f * c.H) && (rn < 1e-8f * c.H)) {
                    if (!self_added) {
                        const float rt = fabsf(dot_d<D>(d, tj));
                        const float rb = fabsf(dot_d<D>(d, bj));
                        const float dr = 0.55f * powf(area, 1.f / (c.DIMS - 1.f));
                        if ((rt <= dr) && (rb <= dr)) {
                            self_added = true;
                            shep = shep - 0.5f;
                        }
                    }
                } else {
                    const float rt = fabsf(dot_d<D>(d, tj));
                    const float rb = fabsf(dot_d<D>(d, bj));
                    shep = shep + (rn * c.CONW * kernel_sp<D>(q) * area +
                                   kernel_sd<D>(fabsf(rn), rt, rb, area));
                }
                if (fluid) {
                    const float pw = a.b.pmq[j].x;
                    const float4 vw = a.b.velq[j];
                    const float w = kernel_w<D>(q) * c.CONW * area;
                    const float sg = (p_i + pw) / rho_i * w;
                    for (int kk = 0; kk < D; kk++)
                        gp[kk] = gp[kk] + sg * nj[kk];
                    float dv[3];
                    dv[0] = vw.x - uiv[0];
                    dv[1] = vw.y - uiv[1];
                    dv[2] = (D == 3) ? vw.z - uiv[2] : 0.f;
                    du = du + rho_i * dot_d<D>(dv, nj) * w;
                }
            }
        }
    }
    if (a.b.shepard)
        a.b.shepard[i] = want_shep ? shep : 0.f;

    float ui_full[4];
    Vec<D>::load(T.u, i, ui_full);  // the velocity the sums used, incl. w
    float gpf[4] = { 0.f, 0.f, 0.f, 0.f }, luf[4] = { 0.f, 0.f, 0.f, 0.f };
    float gwf[4] = { 0.f, 0.f, 0.f, 0.f };
    float div_u = 0.f;
    if (fluid && bie) {
        for (int k = 0; k < D; k++) {
            gpf[k] = gp[k];
            luf[k] = lu[k];
            gwf[k] = gw[k];
        }
        // BIe Rates.cl
        const float s2 = 2.f * p_i / rho_i;
        for (int k = 0; k < VS; k++)
            gpf[k] = gpf[k] + s2 * gwf[k];
        div_u = du - 2.f * rho_i * (dot_full<D>(ui_full, gwf) + dbi);
    } else if (fluid) {
        // BI/Shepard.cl apply: renormalise by the analytic Shepard factor
        for (int k = 0; k < D; k++) {
            gpf[k] = gp[k];
            luf[k] = lu[k];
        }
        for (int k = 0; k < VS; k++) {
            gpf[k] = gpf[k] / shep;
            luf[k] = luf[k] / shep;
        }
        div_u = du / shep;
    }
    if (a.extras) {
        Vec<D>::store(a.b.grad_p, i, gpf);
        Vec<D>::store(a.b.lap_u, i, luf);
        Vec<D>::store(a.b.grad_w_bi, i, gwf);
        a.b.div_u[i] = div_u;
        a.b.lap_p[i] = fluid ? lp : 0.f;
        a.b.div_u_bi[i] = fluid ? dbi : 0.f;
    }

    if (sensor) {
        float shp = shep;
        if (shp < 1.0e-6f)
            shp = 1.f;
        float uo[4];
        for (int k = 0; k < 4; k++)
            uo[k] = ui_full[k];
        for (int k = 0; k < D; k++)
            uo[k] = gp[k];
        for (int k = 0; k < VS; k++)
            uo[k] = uo[k] / shp;
        Vec<D>::store(T.u, i, uo);
        T.rho[i] = du / shp;
        T.p[i] = lp / shp;
    }

    if (im <= 0)
        return c.dt_fixed;

    const uint32_t set_raw = T.iset[i];
    const uint32_t set = set_raw < c.n_sets ? set_raw : 0u;
    float acc[4];
    float drhodt;
    float ain[4];
    Vec<D>::load(a.b.dudt_in, i, ain);
    const float drhodt_in = a.b.drhodt_in[i];
    float uin[4] = { 0.f, 0.f, 0.f, 0.f };
    Vec<D>::load(a.b.u_in, i, uin);
    if (fluid) {
        // cfd Rates.cl + deltaSPH
        const float visc = c.visc_dyn[set];
        for (int k = 0; k < VS; k++)
            acc[k] = -gpf[k] + visc * luf[k] + c.g[k];
        drhodt = -div_u;
        const float delta_f = c.delta[set] * dt * rho_i / c.refd[set];
        drhodt = drhodt + delta_f * lp;
        // BIe ElasticBounce.cl
        if (bie && dt != 0.f) {
            float vh[3];
            for (int k = 0; k < D; k++)
                vh[k] = uin[k] + hdt * acc[k];
            for (int k = 0; k < NC; k++) {
                const uint32_t cn = neighbour_cell<D>(key_i, k, nx, nxy);
                const uint2 se = a.b.wall_range[cn];  // empty: x > y
                for (uint32_t j = se.x; j < se.y; j++) {
                    const float4 pj = a.b.posq[j];
                    if (__float_as_int(pj.w) != -3)
                        continue;
                    float d[3], nj[3], t[3];
                    d[0] = pj.x - ri[0];
                    d[1] = pj.y - ri[1];
                    d[2] = (D == 3) ? pj.z - ri[2] : 0.f;
                    load_normal<D>(a.dst.normal, j, nj);
                    const float rn = dot_d<D>(d, nj);
                    if (rn < 0.f)
                        continue;
                    const float mj = a.b.pmq[j].y;
                    const float dr = (D == 3) ? sqrtf(mj) : mj;
                    const float R = c.dr_factor * dr;
                    for (int kk = 0; kk < D; kk++)
                        t[kk] = d[kk] - rn * nj[kk];
                    if (dot_d<D>(t, t) >= R * R)
                        continue;
                    const float drn = dt * dot_d<D>(vh, nj);
                    if (drn < 0.f)
                        continue;
                    if (rn - drn <= c.min_bound_dist * dr) {
                        float v[3], vr[3];
                        for (int kk = 0; kk < D; kk++)
                            v[kk] = uin[kk] + dt * acc[kk];
                        const float vn2 = 2.f * dot_d<D>(v, nj);
                        for (int kk = 0; kk < D; kk++)
                            vr[kk] = v[kk] - vn2 * nj[kk];
                        for (int kk = 0; kk < D; kk++) {
                            acc[kk] = (vr[kk] - uin[kk]) / dt;
                            vh[kk] = uin[kk] + hdt * acc[kk];
                        }
                    }
                }
            }
        }
    } else {
        // no rates computed: the Variables keep what k_gather left there
        // (the sorted old rates under midpoint)
        Vec<D>::load(T.dudt, i, acc);
        drhodt = T.drhodt[i];
    }
    float rin[4] = { 0.f, 0.f, 0.f, 0.f };
    Vec<D>::load(a.b.r_in, i, rin);
    float rn_[4] = { 0.f, 0.f, 0.f, 0.f }, un[4] = { 0.f, 0.f, 0.f, 0.f };
    float rho_n;
    if (c.scheme == AQUA_SCHEME_IMPROVED_EULER) {
        // improved_euler.cl corrector: r_in, u_in, rho_in hold the sorted
        // predictor output
        const float DT = 0.5f * dt;
        const float DT2 = DT * DT;
        for (int k = 0; k < VS; k++) {
            const float da = acc[k] - ain[k];
            un[k] = uin[k] + DT * da;
            rn_[k] = rin[k] + DT2 * da;
        }
        rho_n = a.b.rho_in[i] + DT * (drhodt - drhodt_in);
    } else {
        // midpoint relax
        const float rl = c.relax_midpoint;
        for (int k = 0; k < VS; k++)
            acc[k] = rl * ain[k] + (1.f - rl) * acc[k];
        drhodt = rl * drhodt_in + (1.f - rl) * drhodt;
        // corrector
        const float hdt2 = 0.5f * dt * dt;
        for (int k = 0; k < VS; k++) {
            rn_[k] = rin[k] + dt * uin[k] + hdt2 * acc[k];
            un[k] = uin[k] + dt * acc[k];
        }
        rho_n = a.b.rho_in[i] + dt * drhodt;
    }
    // BIe PST.cl
    if (fluid && bie) {
        const float Ri = 0.5f * powf(T.m[i] / rho_n, 1.f / c.DIMS);
        for (int k = 0; k < NC; k++) {
            const uint32_t cn = neighbour_cell<D>(key_i, k, nx, nxy);
            const uint2 se = a.b.wall_range[cn];  // empty: x > y
            for (uint32_t j = se.x; j < se.y; j++) {
                const float4 pj = a.b.posq[j];
                if (__float_as_int(pj.w) != -3)
                    continue;
                float d[3], nj[3], t[3];
                d[0] = pj.x - rn_[0];
                d[1] = pj.y - rn_[1];
                d[2] = (D == 3) ? pj.z - rn_[2] : 0.f;
                load_normal<D>(a.dst.normal, j, nj);
                const float rn = dot_d<D>(d, nj);
                if (fabsf(rn) > Ri)
                    continue;
                const float mj = a.b.pmq[j].y;
                const float dr = (D == 3) ? sqrtf(mj) : mj;
                const float Rj = c.dr_factor * dr;
                for (int kk = 0; kk < D; kk++)
                    t[kk] = d[kk] - rn * nj[kk];
                if (dot_d<D>(t, t) >= Rj * Rj)
                    continue;
                const float sh = rn - Ri;
                for (int kk = 0; kk < D; kk++)
                    rn_[kk] = rn_[kk] + sh * nj[kk];
            }
        }
    }
    Vec<D>::store(T.dudt, i, acc);
    T.drhodt[i] = drhodt;
    Vec<D>::store(T.r, i, rn_);
    Vec<D>::store(T.u, i, un);
    T.rho[i] = rho_n;
    // TimeStep.cl
    const float dr_max = c.dt_Ma * c.h;
    const float dt_u = c.courant * dr_max / sqrtf(dot_full<D>(un, un));
    return cl_max(cl_min(c.dt_fixed, dt_u), c.dt_min);
}

// Persistent sweep: warps fetch cell-aligned chunks of <= 32 particles
// NT threads per block, NQ queued neighbours per thread (power of 2, >= 64)
// of type QE, candidate groups copied by the bulk-copy engine when BULK,
// BI walls (cfd/BI.xml) when BI, else BIe walls
template<int D, int NT, int NQ, typename QE, bool BULK, bool BI, int MODE,
         int MINW = 20>
__global__ void __launch_bounds__(NT, MINW * 32 / NT)
k_sweep(Consts c, StepArgs a)
{
    // per-lane queues, or (direct) per warp the velocity/density and
    // pressure/mass records of the current candidate group (two buffers each
    // when the groups are prefetched)
    constexpr int WP = (MODE == kSweepQueue) ? 1 : NT / 32;
    __shared__ QE s_queue[MODE == kSweepQueue ? NQ * NT : 1];
    __shared__ __align__(16) float4 s_vel[WP][2 * 32];
    __shared__ __align__(8) float2 s_pm[WP][2 * 32];
    __shared__ float s_box[NT / 32][8];
    __shared__ uint32_t s_cstart[NT / 32][32];
    __shared__ __align__(16) float4 s_grp[NT / 32][2 * 32];
    __shared__ __align__(8) uint64_t s_mbar[NT / 32][2];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x < (NT / 32) * 2) {
        const uint32_t mb = (uint32_t)__cvta_generic_to_shared(
            &s_mbar[threadIdx.x >> 1][threadIdx.x & 1]);
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(mb));
    }
    __syncthreads();
    uint32_t phases = 0;  // parity of the next completion of each buffer
    // running minimum of dt_var of the warp's current case, flushed to the
    // case's dt_next when the case changes and at the end
    float run_min = INFINITY;
    uint32_t run_case = 0xffffffffu;
    auto flush = [&]() {
        if (lane == 0 && run_case != 0xffffffffu) {
            if (run_min < INFINITY && run_min >= 0.f)
                atomicMin(&a.cs[run_case].dt_next, __float_as_uint(run_min));
            else if (!(run_min >= 0.f))
                atomicOr(&a.sc->err, kErrDt);
        }
    };
    if (a.sc->err == 0) {
        const uint32_t nch = a.sc->n_chunks;
        for (;;) {
            uint32_t ch = 0;
            if (lane == 0)
                ch = atomicAdd(&a.sc->chunk_next, 1u);
            ch = __shfl_sync(0xffffffffu, ch, 0);
            if (ch >= nch)
                break;
            const uint2 cw = a.b.chunks[ch];
            const bool valid = (uint32_t)lane < cw.y;
            float v = sweep_particle<D, NT, NQ, QE, BULK, BI, MODE>(
                c, a, valid ? cw.x + lane : cw.x, valid,
                s_queue + (MODE == kSweepQueue ? threadIdx.x : 0),
                s_cstart[warp], s_grp[warp], s_mbar[warp], phases,
                s_vel[WP > 1 ? warp : 0], s_pm[WP > 1 ? warp : 0],
                s_box[warp]);
            __syncwarp();  // s_cstart and s_grp are rewritten for the next chunk
            for (int o = 16; o > 0; o >>= 1)
                v = cl_min(v, __shfl_xor_sync(0xffffffffu, v, o));
            const uint32_t kc = a.dst.cid[cw.x];
            if (kc != run_case) {
                flush();
                run_case = kc;
                run_min = INFINITY;
            }
            run_min = cl_min(run_min, v);
        }
    }
    flush();
}

// BI walls before the sweep (cfd/BI.xml): for every boundary element, its
// analytic Shepard factor (BI/Shepard.cl compute: the other elements of the
// support), the free-slip Laplacian of the fluid velocity (BI/LapU.cl), the
// pressure gradient it implies (BI/GradP.cl), the pressure interpolated
// from the fluid (BI/Interpolation.cl, a second pass: it needs that
// gradient) and its Shepard renormalisation with the density from the
// linear EOS (BI/InterpolationShepard.cl).  The sweep then reads the
// elements' pressure from the packed records.
template<int D>
__global__ void __launch_bounds__(128)
k_bi_walls(Consts c, StepArgs a)
{
    constexpr int VS = Vec<D>::VS;
    constexpr int NC = (D == 3) ? 27 : 9;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.N || a.sc->err)
        return;
    const float4 pi = a.b.posq[i];
    if (__float_as_int(pi.w) != -3)
        return;
    const VarSet& T = a.dst;
    const CaseScalars& cas = a.cs[T.cid[i]];
    const uint32_t nx = cas.n_cells[0];
    const uint32_t nxy = cas.n_cells[0] * cas.n_cells[1];
    const uint32_t key_i = a.skeys[i];
    const float ri[3] = { pi.x, pi.y, pi.z };
    const float4 vi = a.b.velq[i];
    const float ui[3] = { vi.x, vi.y, vi.z };
    float shep = 1.f;
    bool self_added = false;
    float lap[4] = { 0.f, 0.f, 0.f, 0.f };
    for (int k = 0; k < NC; k++) {
        const uint2 se = a.b.cells[neighbour_cell<D>(key_i, k, nx, nxy)];
        for (uint32_t j = se.x; j < se.y; j++) {
            const float4 pj = a.b.posq[j];
            const int jm = __float_as_int(pj.w);
            if (jm == -3) {
                if (j == i) {
                    if (!self_added) {
                        self_added = true;
                        shep = shep - 0.5f;
                    }
                    continue;
                }
            } else if (jm != 1) {
                continue;
            }
            float d[3];
            d[0] = pj.x - ri[0];
            d[1] = pj.y - ri[1];
            d[2] = (D == 3) ? pj.z - ri[2] : 0.f;
            const float q = sqrtf(dot_d<D>(d, d)) / c.H;
            if (q >= c.SUPPORT)
                continue;
            if (jm == 1) {
                const float4 vj = a.b.velq[j];
                const float f = kernel_f<D>(q) * c.CONF * a.b.pmq[j].y;
                const float s2 = f * 2.f / vj.w;
                lap[0] = lap[0] + s2 * (vj.x - ui[0]);
                lap[1] = lap[1] + s2 * (vj.y - ui[1]);
                if (D == 3)
                    lap[2] = lap[2] + s2 * (vj.z - ui[2]);
                continue;
            }
            float nj[3], tj[3], bj[3];
            load_normal<D>(T.normal, j, nj);
            load_normal<D>(T.tangent, j, tj);
            load_normal<D>(T.binormal, j, bj);
            const float area = a.b.pmq[j].y;
            const float rn = dot_d<D>(d, nj);
            if ((rn > -1e-8f * c.H) && (rn < 1e-8f * c.H)) {
                if (!self_added) {
                    const float rt = fabsf(dot_d<D>(d, tj));
                    const float rb = fabsf(dot_d<D>(d, bj));
                    const float dr = 0.55f * powf(area, 1.f / (c.DIMS - 1.f));
                    if ((rt <= dr) && (rb <= dr)) {
                        self_added = true;
                        shep = shep - 0.5f;
                    }
                }
                continue;
            }
            const float rt = fabsf(dot_d<D>(d, tj));
            const float rb = fabsf(dot_d<D>(d, bj));
            shep = shep + (rn * c.CONW * kernel_sp<D>(q) * area +
                           kernel_sd<D>(fabsf(rn), rt, rb, area));
        }
    }
    // BI/GradP.cl freeslip
    const uint32_t set_raw = T.iset[i];
    const uint32_t set = set_raw < c.n_sets ? set_raw : 0u;
    const float sh = shep < 1.0e-6f ? 1.f : shep;
    // the dudt Variable: the sorted old rates (midpoint init copy) or, under
    // improved Euler, the unpermuted array (see k_gather)
    float dudt[4];
    Vec<D>::load(T.dudt, i, dudt);
    float gw[4];
    for (int k = 0; k < VS; k++)
        gw[k] = c.visc_dyn[set] / c.refd[set] * lap[k] / sh + c.g[k] - dudt[k];
    // BI/Interpolation.cl
    const float rho_i = vi.w;
    float gpi[3];
    for (int k = 0; k < 3; k++)
        gpi[k] = rho_i * gw[k];
    float p = 0.f;
    for (int k = 0; k < NC; k++) {
        const uint2 se = a.b.cells[neighbour_cell<D>(key_i, k, nx, nxy)];
        for (uint32_t j = se.x; j < se.y; j++) {
            const float4 pj = a.b.posq[j];
            if (__float_as_int(pj.w) != 1)
                continue;
            float d[3];
            d[0] = pj.x - ri[0];
            d[1] = pj.y - ri[1];
            d[2] = (D == 3) ? pj.z - ri[2] : 0.f;
            const float q = sqrtf(dot_d<D>(d, d)) / c.H;
            if (q >= c.SUPPORT)
                continue;
            const float2 pm = a.b.pmq[j];
            const float w = kernel_w<D>(q) * c.CONW * pm.y / a.b.velq[j].w;
            p = p + (pm.x - dot_d<D>(gpi, d)) * w;
        }
    }
    // BI/InterpolationShepard.cl
    p = p / sh;
    const float rho = c.refd[set] + (p - c.p0) / (c.cs * c.cs);
    T.p[i] = p;
    T.rho[i] = rho;
    a.b.pmq[i].x = p;
    if (a.b.shepard)
        a.b.shepard[i] = shep;
    if (a.extras) {
        Vec<D>::store(a.b.lap_u, i, lap);
        Vec<D>::store(a.b.grad_p, i, gw);
    }
}

template<int D>
cudaError_t
launch_bi_walls_impl(const Consts& c, const StepArgs& a, cudaStream_t s)
{
    if (a.N == 0)
        return cudaSuccess;
    k_bi_walls<D><<<(a.N + 127) / 128, 128, 0, s>>>(c, a);
    return cudaGetLastError();
}

template<int D>
cudaError_t
launch_gather_impl(const Consts& c, const StepArgs& a, cudaStream_t s)
{
    if (a.N == 0)
        return cudaSuccess;
    k_gather<D><<<(a.N + 255) / 256, 256, 0, s>>>(c, a);
    return cudaGetLastError();
}

// sweep variants the tuner chooses from: (threads per block, queue depth,
// queue entry type, bulk-copy staging) for the queued sweep, or threads per
// block for the direct one; a block's static shared memory stays <= 37 KB
template<int D>
cudaError_t
launch_sweep_impl(const Consts& c, const StepArgs& a, unsigned grid,
                  int variant, cudaStream_t s)
{
    if (a.N == 0)
        return cudaSuccess;
    if (c.boundary == AQUA_BOUNDARY_BI) {
        // one launch shape for the BI walls: the direct sweep with prefetch
        // and the register budget of 28 resident warps per SM
        k_sweep<D, 64, 1, uint32_t, true, true, kSweepDirect, 28><<<grid, 64, 0, s>>>(c, a);
        return cudaGetLastError();
    }
    switch (variant) {
    case 1:
        k_sweep<D, 64, 128, uint16_t, false, false, kSweepQueue><<<grid, 64, 0, s>>>(c, a);
        break;
    case 2:
        k_sweep<D, 64, 64, uint32_t, false, false, kSweepQueue><<<grid, 64, 0, s>>>(c, a);
        break;
    case 3:
        k_sweep<D, 64, 128, uint16_t, true, false, kSweepQueue><<<grid, 64, 0, s>>>(c, a);
        break;
    case 4:
        k_sweep<D, 64, 64, uint32_t, true, false, kSweepQueue><<<grid, 64, 0, s>>>(c, a);
        break;
    case 5:
        k_sweep<D, 64, 1, uint32_t, false, false, kSweepDirect><<<grid, 64, 0, s>>>(c, a);
        break;
    case 6:
        k_sweep<D, 128, 1, uint32_t, false, false, kSweepDirect><<<grid, 128, 0, s>>>(c, a);
        break;
    case 7:
        k_sweep<D, 64, 1, uint32_t, true, false, kSweepDirect><<<grid, 64, 0, s>>>(c, a);
        break;
    case 8:
        k_sweep<D, 128, 1, uint32_t, true, false, kSweepDirect><<<grid, 128, 0, s>>>(c, a);
        break;
    // the same with the register budget of 28, 32 or 36 resident warps per
    // SM
    case 9:
        k_sweep<D, 64, 1, uint32_t, true, false, kSweepDirect, 28><<<grid, 64, 0, s>>>(c, a);
        break;
    case 10:
        k_sweep<D, 128, 1, uint32_t, true, false, kSweepDirect, 28><<<grid, 128, 0, s>>>(c, a);
        break;
    case 11:
        k_sweep<D, 64, 1, uint32_t, true, false, kSweepDirect, 32><<<grid, 64, 0, s>>>(c, a);
        break;
    case 12:
        k_sweep<D, 128, 1, uint32_t, true, false, kSweepDirect, 32><<<grid, 128, 0, s>>>(c, a);
        break;
    case 13:
        k_sweep<D, 64, 1, uint32_t, true, false, kSweepDirect, 36><<<grid, 64, 0, s>>>(c, a);
        break;
    case 14:
        k_sweep<D, 128, 1, uint32_t, true, false, kSweepDirect, 36><<<grid, 128, 0, s>>>(c, a);
        break;
    default:
        k_sweep<D, 128, 128, uint16_t, false, false, kSweepQueue><<<grid, 128, 0, s>>>(c, a);
        break;
    }
    return cudaGetLastError();
}

template cudaError_t launch_bi_walls_impl<2>(const Consts&, const StepArgs&, cudaStream_t);
template cudaError_t launch_bi_walls_impl<3>(const Consts&, const StepArgs&, cudaStream_t);
template cudaError_t launch_gather_impl<2>(const Consts&, const StepArgs&, cudaStream_t);
template cudaError_t launch_gather_impl<3>(const Consts&, const StepArgs&, cudaStream_t);
template cudaError_t launch_sweep_impl<2>(const Consts&, const StepArgs&, unsigned,
                                          int, cudaStream_t);
template cudaError_t launch_sweep_impl<3>(const Consts&, const StepArgs&, unsigned,
                                          int, cudaStream_t);
