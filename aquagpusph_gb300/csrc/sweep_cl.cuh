// The clustered neighbour sweep of the fast build (3-D, BIe walls, midpoint
// scheme): the same sums, rates and integrator as k_sweep
// (cfd/Interactions.cl:60-145, basic/Shepard.cl:76-125, cfd/Sensors.cl,
// basic/deltaSPH.cl:191-242,330-350, BIe/{Interactions,Rates,ElasticBounce,
// PST}.cl, cfd/Rates.cl, midpoint.cl corrector, cfd/TimeStep.cl), with the
// pair work laid out so that most lanes do useful arithmetic.
//
// Work unit: a cell.  A block of NW warps takes the next cell from a work
// counter and stages the packed records (rec0, rec1: 32 B per particle) of
// its 3^3-cell neighbourhood into shared memory with bulk copies (the TMA
// engine, `cp.async.bulk`, completion on an mbarrier).  The neighbourhood is
// nine contiguous runs of sorted particles (one per (dy, dz) row: the cell
// keys run x-fastest).
//
// Clusters: k_clusters groups each cell's particles by octant into
// clusters of at most 8 (small octant groups merge).  A warp takes one
// cluster at a time as 8 particles x 4 neighbour slots: lane l holds
// particle l % 8 and takes every fourth neighbour of the cluster's list from
// slot l / 8 on, so that the 8 lanes of one phase of a 16-byte shared load
// read the same record (a broadcast, free of bank conflicts).
// The list holds the staged candidates within the support of the octant
// boxes of the cluster's particles.  After each staging the block
// classifies every staged record once into a 16-bit mask: the octant boxes
// of the cell it comes within the support of (a box per octant, spanning,
// per axis and half, the cell's particles there), in the low byte for a
// fluid record and the high byte for a boundary element.  Each cluster then
// scans those masks and compacts its candidates with ballots.  About 60% of the evaluated pairs lie in the support on a
// lattice, against about a third of the lanes in k_sweep.  Pairs outside
// the support add exact zeros (the kernel factor is cut to zero at
// q >= SUPPORT), so the lists only have to be conservative: each octant
// box holds its particles.  The four partial sums of a particle are added
// by two butterfly shuffles.
//
// Summation order differs from the reference's (neighbours in staging
// order, four interleaved partial sums): this sweep is the fast build's,
// checked within the per-step rate tolerance 1e-5.  It is deterministic:
// clusters, lists and staging depend on the sorted state only, not on the
// launch shape.
//
// Boundary elements reach fluid particles through a second list (the BIe
// wall sums), which also serves the elastic bounce and PST of the
// epilogue.  Where that list overflowed or the neighbourhood needed more
// than one staging pass, the epilogue walks the boundary elements of the
// 27 cells from global memory instead (the per-cell index ranges of k_gather).
//
// Probes (imove 0) form clusters of their own; each lane of a probe cluster
// sums its probe's neighbours in a plain loop over the staged records.
//
// With a rate sample (aqua_set_rate_sample) only the cells whose key hashes
// below the sample's threshold, and the cells around a probe, are swept;
// the other particles keep what k_gather wrote.
//
// This header is included by step_fast.cu only, inside namespace aqua::fast.

namespace {

constexpr int kClListCap = 192;      // fluid survivors per warp (128 per round
                                     // of the mask scan, drained above 64)
constexpr int kClWallCap = 192;      // boundary-element survivors per warp
// per staged record: bit o (o < 8) of a fluid record, bit 8 + o of a
// boundary element = within the support of the cell's octant box o
constexpr uint32_t kMaskWallShift = 8;
constexpr int kClMaxPieces = 32;     // staged runs per pass
constexpr uint32_t kClWaitLimit = 1u << 22;

// Shared memory of one block: staged records (CAP + 1: the last is a zero
// record that pads the lists to whole quads), per-warp lists, staged runs
template<int NW, int CAP>
struct ClSmem
{
    float4 r0[CAP + 1];
    float4 r1[CAP + 1];
    uint16_t list[NW][kClListCap + 4];   // + room for the padding quad
    uint16_t wall[NW][kClWallCap + 4];
    // the staged boundary elements, by warp-sized chunks of the staging
    alignas(8) uint16_t mask[CAP + 4];  // per staged record: octants by kind
    float ivl[12];               // octant boxes: axis a, half h: [lo, hi] at 4 a + 2 h
    uint4 piece[kClMaxPieces];   // (slot, sorted first, count, -)
    uint2 row[9];                // (sorted first, count) of each row
    uint32_t npieces;
    uint32_t nstaged;
    uint32_t total;              // candidates of the neighbourhood
    uint32_t work;
    uint64_t mbar;
};

// Octant (0-7, x fastest) of a position inside its cell: the halves of the
// cell along each axis (cells are (support h) wide from the case's r_min)
__device__ __forceinline__ uint32_t
cl_octant(const float4 p, const CaseScalars& cs, float sc2)
{
    const uint32_t ox = (uint32_t)((p.x - cs.r_min[0]) * sc2) & 1u;
    const uint32_t oy = (uint32_t)((p.y - cs.r_min[1]) * sc2) & 1u;
    const uint32_t oz = (uint32_t)((p.z - cs.r_min[2]) * sc2) & 1u;
    return ox | (oy << 1) | (oz << 2);
}

// The cells holding particles, as (key, first sorted index), and their
// (first, end, -, case) in the cluster table: position s starts a cell
// where the sorted key changes.  A block takes
// kCellListThreads x kCellListItems positions and reserves its entries with
// one atomicAdd (the order of the list does not matter: every cell is swept
// the same wherever it sits in it).
constexpr int kCellListThreads = 1024;
constexpr int kCellListItems = 8;
__global__ void __launch_bounds__(kCellListThreads)
k_cell_list(const uint32_t* skeys, uint32_t N, const uint2* cells,
            const uint32_t* cid, uint2* work, uint4* wcl, DevScalars* sc)
{
    __shared__ uint32_t s_warp[kCellListThreads / 32];
    __shared__ uint32_t s_base;
    if (__syncthreads_or(threadIdx.x == 0 && sc->err))
        return;  // one read for the whole block
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t base = blockIdx.x * (uint32_t)(kCellListThreads * kCellListItems);
    uint32_t starts = 0;  // bit it: position base + it * threads + t starts a cell
    for (int it = 0; it < kCellListItems; it++) {
        const uint32_t s = base + it * kCellListThreads + threadIdx.x;
        if (s < N && (s == 0 || skeys[s - 1] != skeys[s]))
            starts |= 1u << it;
    }
    // block-wide exclusive scan of the counts
    const uint32_t v = (uint32_t)__popc(starts);
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o)
            x += y;
    }
    if (lane == 31)
        s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = s_warp[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o)
                w += y;
        }
        s_warp[lane] = w;  // inclusive warp totals
        if (lane == 31)
            s_base = w ? atomicAdd(&sc->n_chunks, w) : 0u;
    }
    __syncthreads();
    uint32_t o = s_base + (warp > 0 ? s_warp[warp - 1] : 0u) + x - v;
    for (int it = 0; it < kCellListItems; it++) {
        if (starts & (1u << it)) {
            const uint32_t s = base + it * kCellListThreads + threadIdx.x;
            const uint32_t key = skeys[s];
            work[o] = make_uint2(key, s);
            // (first, end, -, case) for k_clusters, which completes it
            wcl[o] = make_uint4(s, cells[key].y, 0u, cid[s]);
            o++;
        }
    }
}

// Clusters of every cell in the work list: one warp per cell.  The cell's
// particles are ordered by group (octants 0-7 of the cell, then probes) into
// cperm[first .. end) and cut into clusters: a group joins the open cluster
// when it fits whole, else it starts new ones of 8 (probes always start a
// new cluster).  Ranks within a group follow the sorted order, so the
// clusters are a function of the sorted state.
__global__ void __launch_bounds__(256)
k_clusters(Consts c, StepArgs a)
{
    __shared__ uint32_t s_cnt[8][16];
    __shared__ uint32_t s_pos[8][16];
    if (a.sc->err)
        return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t n_work = a.sc->n_chunks;
    const uint32_t lt = (1u << lane) - 1u;
    for (uint32_t w = blockIdx.x * 8u + warp; w < n_work; w += gridDim.x * 8u) {
        const uint4 wc0 = a.b.wcl[w];  // (first, end, -, case) of k_cell_list
        const uint32_t first = wc0.x;
        const uint32_t end = wc0.y;
        const uint32_t n = end - first;
        const CaseScalars& cs = a.cs[wc0.w];
        // row (dy, dz) = (lane % 3 - 1, lane / 3 - 1) of the sweep's
        // neighbourhood: cells x-1 .. x+1, as one run of sorted indices
        // (lanes 0-8; the cell table is read here and the row written after
        // the clusters, so the loads overlap the work below)
        uint2 rc3[3] = { make_uint2(1u, 0u), make_uint2(1u, 0u), make_uint2(1u, 0u) };
        if (lane < 9) {
            const uint32_t key = a.b.work[w].x;
            const uint32_t nx = cs.n_cells[0];
            const uint32_t nxy = cs.n_cells[0] * cs.n_cells[1];
            const uint32_t k0 = key + (uint32_t)(lane % 3 - 1) * nx +
                                (uint32_t)(lane / 3 - 1) * nxy - 1u;
            for (int d = 0; d < 3; d++)
                rc3[d] = a.b.cells[k0 + d];
        }
        const float sc2 = 2.f * c.idist;
        auto group = [&](uint32_t s) -> uint32_t {
            if (a.dst.imove[s] == 0)
                return 8u;
            return cl_octant(a.b.rec0[s], cs, sc2);
        };
        if (lane < 16)
            s_cnt[warp][lane] = 0;
        __syncwarp();
        for (uint32_t b = 0; b < n; b += 32) {
            const bool v = b + lane < n;
            const uint32_t g = v ? group(first + b + lane) : 16u;
            const unsigned m = __match_any_sync(0xffffffffu, g);
            if (v && lane == __ffs(m) - 1)
                s_cnt[warp][g] += (uint32_t)__popc(m);
            __syncwarp();
        }
        if (lane == 0) {
            // the walk over the groups: counts the clusters, then writes them
            auto walk = [&](bool write, uint32_t k) -> uint32_t {
                uint32_t pos = 0, coff = 0, ccnt = 0;
                bool open = false;
                for (uint32_t g = 0; g < 9; g++) {
                    const uint32_t cg = s_cnt[warp][g];
                    if (write)
                        s_pos[warp][g] = pos;
                    if (cg == 0)
                        continue;
                    if (open && (g == 8 || ccnt + cg > 8)) {
                        if (write)
                            a.b.clu[k] = make_uint2(first + coff, ccnt);
                        k++;
                        open = false;
                    }
                    if (open) {
                        ccnt += cg;
                    } else {
                        uint32_t left = cg, p = pos;
                        while (left > 8) {
                            if (write)
                                a.b.clu[k] = make_uint2(first + p, 8u);
                            k++;
                            p += 8;
                            left -= 8;
                        }
                        coff = p;
                        ccnt = left;
                        open = true;
                    }
                    pos += cg;
                }
                if (open) {
                    if (write)
                        a.b.clu[k] = make_uint2(first + coff, ccnt);
                    k++;
                }
                return k;
            };
            // a cell has at most as many clusters as particles: its
            // clusters take the slots of clu from its first sorted index on
            const uint32_t n_cl = walk(true, first) - first;
            a.b.wcl[w] = make_uint4(first, end, wc0.w, n_cl);
        }
        __syncwarp();
        if (lane < 16)
            s_cnt[warp][lane] = 0;  // running ranks
        __syncwarp();
        for (uint32_t b = 0; b < n; b += 32) {
            const bool v = b + lane < n;
            const uint32_t s = first + b + lane;
            const uint32_t g = v ? group(s) : 16u;
            const unsigned m = __match_any_sync(0xffffffffu, g);
            if (v)
                a.b.cperm[first + s_pos[warp][g] + s_cnt[warp][g] +
                          (uint32_t)__popc(m & lt)] = s;
            __syncwarp();
            if (v && lane == __ffs(m) - 1)
                s_cnt[warp][g] += (uint32_t)__popc(m);
            __syncwarp();
        }
        if (lane < 9) {
            uint32_t lo = 0xffffffffu, hi = 0;
            for (int d = 0; d < 3; d++) {
                if (rc3[d].x < rc3[d].y) {
                    lo = min(lo, rc3[d].x);
                    hi = max(hi, rc3[d].y);
                }
            }
            a.b.crow[(size_t)w * 9 + lane] = hi > lo ? make_uint2(lo, hi - lo) : make_uint2(0u, 0u);
        }
    }
}


// Everything after the sums for sorted particle i of a cluster (the same
// steps and expressions as the epilogue of k_sweep): Shepard, the BIe and
// cfd rates, delta-SPH, elastic bounce, midpoint relax and corrector, PST,
// the variable time step; returns dt_var (+inf for a lane without a
// particle).  The four lanes of a particle compute alike; `store` selects
// the one that writes.  The boundary elements of the elastic bounce and the
// PST come from the cluster's staged wall list (entries wl[0 .. wfill) of
// the staged records) or, when `walls_global`, from the per-cell index
// ranges of the 27 cells around `key` in global memory.
__device__ __forceinline__ float
sweep_cl_finish(const Consts& c, const StepArgs& a, uint32_t i, bool valid,
                int im, bool want, bool fluid, bool sensor, bool store,
                float dt, const float4 r0i, const float4 r1i, float shep,
                float gp0, float gp1, float gp2, float lu0, float lu1,
                float lu2, float du, float lp, float gw0, float gw1, float gw2,
                float dbi, bool walls_global, const uint16_t* wl,
                uint32_t wfill, const float4* sr0, const float4* sr1,
                uint32_t key, const CaseScalars& cas)
{
    if (!valid)
        return INFINITY;
    const VarSet& T = a.dst;
    const float hdt = 0.5f * dt;
    const float p_i = r1i.w;
    if (store && a.b.shepard)
        a.b.shepard[i] = want ? shep : 0.f;
    float ain[4], uin[4];
    Vec<3>::load(a.b.dudt_in, i, ain);
    Vec<3>::load(a.b.u_in, i, uin);
    const float drhodt_in = a.b.drhodt_in[i];
    // the midpoint density and velocity of k_gather: recomputed for fluid
    // (the gather leaves T.rho and T.u to this epilogue), read otherwise
    float rho_i, ui_full[4];
    if (fluid) {
        rho_i = a.b.rho_in[i] + hdt * drhodt_in;
        for (int k = 0; k < 4; k++)
            ui_full[k] = uin[k] + hdt * ain[k];
    } else {
        rho_i = T.rho[i];
        const float4 u4 = reinterpret_cast<const float4*>(T.u)[i];
        ui_full[0] = u4.x;
        ui_full[1] = u4.y;
        ui_full[2] = u4.z;
        ui_full[3] = u4.w;
    }
    float gpf[4] = { 0.f, 0.f, 0.f, 0.f }, luf[4] = { 0.f, 0.f, 0.f, 0.f };
    float gwf[4] = { 0.f, 0.f, 0.f, 0.f };
    float div_u = 0.f;
    if (fluid) {
        // the factors left out of the pair sums: those of particle i, and
        // CONF F-factor / (CONW W-factor) (the staged volumes carry the
        // latter)
        const float kf = c.f_over_w;
        const float ir = kf / rho_i;
        const float ir2 = 2.f * ir;
        gpf[0] = gp0 * ir;
        gpf[1] = gp1 * ir;
        gpf[2] = gp2 * ir;
        luf[0] = lu0 * ir2;
        luf[1] = lu1 * ir2;
        luf[2] = lu2 * ir2;
        du = du * kf;
        lp = lp * kf;
        gwf[0] = gw0;
        gwf[1] = gw1;
        gwf[2] = gw2;
        // BIe Rates.cl
        const float s2 = 2.f * p_i / rho_i;
        for (int k = 0; k < 4; k++)
            gpf[k] = gpf[k] + s2 * gwf[k];
        div_u = du * rho_i - 2.f * rho_i * (dot_full<3>(ui_full, gwf) + dbi);
    }
    if (store && a.extras) {
        Vec<3>::store(a.b.grad_p, i, gpf);
        Vec<3>::store(a.b.lap_u, i, luf);
        Vec<3>::store(a.b.grad_w_bi, i, gwf);
        a.b.div_u[i] = div_u;
        a.b.lap_p[i] = fluid ? lp : 0.f;
        a.b.div_u_bi[i] = fluid ? dbi : 0.f;
    }
    if (sensor) {
        // cfd/SensorsRenormalization.cl
        float shp = shep;
        if (shp < 1.0e-6f)
            shp = 1.f;
        float uo[4] = { gp0, gp1, gp2, ui_full[3] };
        for (int k = 0; k < 4; k++)
            uo[k] = uo[k] / shp;
        if (store) {
            Vec<3>::store(T.u, i, uo);
            T.rho[i] = du / shp;
            T.p[i] = lp / shp;
        }
    }
    if (im <= 0)
        return c.dt_fixed;

    // boundary elements for the elastic bounce and the PST: f(position,
    // normal, area); returns early when f returns true
    const uint32_t nx = cas.n_cells[0];
    const uint32_t nxy = cas.n_cells[0] * cas.n_cells[1];
    auto for_walls = [&](auto&& f) {
        if (!walls_global) {
            for (uint32_t k = 0; k < wfill; k++) {
                const uint32_t j = wl[k];
                const float4 pj = sr0[j];
                const float4 nj = sr1[j];
                f(pj, nj, -pj.w);
            }
            return;
        }
        for (int k = 0; k < 27; k++) {
            const uint32_t cn = neighbour_cell<3>(key, k, nx, nxy);
            const uint2 se = a.b.wall_range[cn];  // empty: x > y
            for (uint32_t j = se.x; j < se.y; j++) {
                const float4 pj = a.b.rec0[j];
                if (!(pj.w < 0.f))
                    continue;
                const float4 nj = a.b.rec1[j];
                f(pj, nj, -pj.w);
            }
        }
    };

    const uint32_t set_raw = T.iset[i];
    const uint32_t set = set_raw < c.n_sets ? set_raw : 0u;
    float acc[4];
    float drhodt;
    const float ri[3] = { r0i.x, r0i.y, r0i.z };
    if (fluid) {
        // cfd Rates.cl + deltaSPH
        const float visc = c.visc_dyn[set];
        for (int k = 0; k < 4; k++)
            acc[k] = -gpf[k] + visc * luf[k] + c.g[k];
        drhodt = -div_u;
        const float delta_f = c.delta[set] * dt * rho_i / c.refd[set];
        drhodt = drhodt + delta_f * lp;
        // BIe ElasticBounce.cl
        if (dt != 0.f) {
            float vh[3];
            for (int k = 0; k < 3; k++)
                vh[k] = uin[k] + hdt * acc[k];
            for_walls([&](const float4 pj, const float4 nj4, float mj) {
                const float nj[3] = { nj4.x, nj4.y, nj4.z };
                float d[3], t[3];
                d[0] = pj.x - ri[0];
                d[1] = pj.y - ri[1];
                d[2] = pj.z - ri[2];
                const float rn = dot_d<3>(d, nj);
                if (rn < 0.f)
                    return;
                const float dr = sqrtf(mj);
                const float R = c.dr_factor * dr;
                for (int kk = 0; kk < 3; kk++)
                    t[kk] = d[kk] - rn * nj[kk];
                if (dot_d<3>(t, t) >= R * R)
                    return;
                const float drn = dt * dot_d<3>(vh, nj);
                if (drn < 0.f)
                    return;
                if (rn - drn <= c.min_bound_dist * dr) {
                    float v[3], vr[3];
                    for (int kk = 0; kk < 3; kk++)
                        v[kk] = uin[kk] + dt * acc[kk];
                    const float vn2 = 2.f * dot_d<3>(v, nj);
                    for (int kk = 0; kk < 3; kk++)
                        vr[kk] = v[kk] - vn2 * nj[kk];
                    for (int kk = 0; kk < 3; kk++) {
                        acc[kk] = (vr[kk] - uin[kk]) / dt;
                        vh[kk] = uin[kk] + hdt * acc[kk];
                    }
                }
            });
        }
    } else {
        Vec<3>::load(T.dudt, i, acc);
        drhodt = T.drhodt[i];
    }
    float rin[4];
    Vec<3>::load(a.b.r_in, i, rin);
    // midpoint relax + corrector
    const float rl = c.relax_midpoint;
    for (int k = 0; k < 4; k++)
        acc[k] = rl * ain[k] + (1.f - rl) * acc[k];
    drhodt = rl * drhodt_in + (1.f - rl) * drhodt;
    float rn_[4], un[4];
    const float hdt2 = 0.5f * dt * dt;
    for (int k = 0; k < 4; k++) {
        rn_[k] = rin[k] + dt * uin[k] + hdt2 * acc[k];
        un[k] = uin[k] + dt * acc[k];
    }
    const float rho_n = a.b.rho_in[i] + dt * drhodt;
    // BIe PST.cl
    if (fluid) {
        const float Ri = 0.5f * powf(T.m[i] / rho_n, 1.f / c.DIMS);
        for_walls([&](const float4 pj, const float4 nj4, float mj) {
            const float nj[3] = { nj4.x, nj4.y, nj4.z };
            float d[3], t[3];
            d[0] = pj.x - rn_[0];
            d[1] = pj.y - rn_[1];
            d[2] = pj.z - rn_[2];
            const float rn = dot_d<3>(d, nj);
            if (fabsf(rn) > Ri)
                return;
            const float dr = sqrtf(mj);
            const float Rj = c.dr_factor * dr;
            for (int kk = 0; kk < 3; kk++)
                t[kk] = d[kk] - rn * nj[kk];
            if (dot_d<3>(t, t) >= Rj * Rj)
                return;
            const float sh = rn - Ri;
            for (int kk = 0; kk < 3; kk++)
                rn_[kk] = rn_[kk] + sh * nj[kk];
        });
    }
    if (store) {
        Vec<3>::store(T.dudt, i, acc);
        T.drhodt[i] = drhodt;
        Vec<3>::store(T.r, i, rn_);
        Vec<3>::store(T.u, i, un);
        T.rho[i] = rho_n;
    }
    // TimeStep.cl
    const float dr_max = c.dt_Ma * c.h;
    const float dt_u = c.courant * dr_max / sqrtf(dot_full<3>(un, un));
    return cl_max(cl_min(c.dt_fixed, dt_u), c.dt_min);
}

__device__ __forceinline__ bool
cl_wait(uint64_t* mbar, uint32_t parity)
{
    const uint32_t mb = (uint32_t)__cvta_generic_to_shared(mbar);
    uint32_t done = 0;
    for (uint32_t it = 0; it < kClWaitLimit && !done; it++)
        asm volatile("{\n.reg .pred p;\n"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                     "selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(done) : "r"(mb), "r"(parity) : "memory");
    return done != 0;
}

// The persistent clustered sweep.  NW warps per block, CAP staged records
// per pass.
template<int NW, int CAP, int MINB>
__global__ void __launch_bounds__(NW * 32, MINB)
k_sweep_cl(Consts c, StepArgs a)
{
    extern __shared__ __align__(128) uint8_t smem_raw[];
    ClSmem<NW, CAP>& S = *reinterpret_cast<ClSmem<NW, CAP>*>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int q = lane >> 3;         // neighbour slot (lanes 8 q .. 8 q + 7)
    const int mq = lane & 7;         // particle of the cluster
    const uint32_t lt = (1u << lane) - 1u;
    const VarSet& T = a.dst;
    if (tid == 0) {
        const uint32_t mb = (uint32_t)__cvta_generic_to_shared(&S.mbar);
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(mb));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        S.r0[CAP] = make_float4(0.f, 0.f, 0.f, 0.f);
        S.r1[CAP] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    uint32_t parity = 0;
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
    const float R2 = c.q2_reject * 1.001f;

    // Stages pass p of the current neighbourhood (the rows' runs as one
    // sequence, CAP records per pass) and waits for it.  Returns false on a
    // time-out (recorded in the error word); every thread returns the same.
    auto stage = [&](uint32_t p) -> bool {
        if (tid == 0) {
            const uint32_t lo = p * (uint32_t)CAP;
            const uint32_t hi = min(S.total, lo + (uint32_t)CAP);
            uint32_t np = 0, off = 0;
            for (int r = 0; r < 9; r++) {
                const uint2 rw = S.row[r];
                const uint32_t a0 = max(off, lo), a1 = min(off + rw.y, hi);
                if (a1 > a0 && np < kClMaxPieces) {
                    S.piece[np++] = make_uint4(a0 - lo, rw.x + (a0 - off), a1 - a0, 0u);
                }
                off += rw.y;
            }
            S.npieces = np;
            S.nstaged = hi - lo;
            const uint32_t mb = (uint32_t)__cvta_generic_to_shared(&S.mbar);
            // the generic reads of the buffers before the async writes
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n"
                         :: "r"(mb), "r"((hi - lo) * 32u) : "memory");
            for (uint32_t k = 0; k < np; k++) {
                const uint4 pc = S.piece[k];
                const uint32_t bytes = pc.z * 16u;
                const uint32_t d0 = (uint32_t)__cvta_generic_to_shared(&S.r0[pc.x]);
                const uint32_t d1 = (uint32_t)__cvta_generic_to_shared(&S.r1[pc.x]);
                const uint64_t g0 = (uint64_t)__cvta_generic_to_global(a.b.rec0 + pc.y);
                const uint64_t g1 = (uint64_t)__cvta_generic_to_global(a.b.rec1 + pc.y);
                asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
                             "[%0], [%1], %2, [%3];\n"
                             :: "r"(d0), "l"(g0), "r"(bytes), "r"(mb) : "memory");
                asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
                             "[%0], [%1], %2, [%3];\n"
                             :: "r"(d1), "l"(g1), "r"(bytes), "r"(mb) : "memory");
            }
        }
        bool ok = cl_wait(&S.mbar, parity);
        if (!ok)
            ok = cl_wait(&S.mbar, parity);  // the copies in flight, again bounded
        else if (c.debug_fake_timeout)
            ok = false;  // test switch: the copies have completed
        parity ^= 1u;
        __syncthreads();  // S.piece / S.nstaged visible; the vote below
        const bool bad = __syncthreads_or(!ok);
        if (bad) {
            if (tid == 0)
                atomicOr(&a.sc->err, kErrTimeout);
            return false;
        }
        // classify the staged records once for all the cell's clusters:
        // their kind, and which octant boxes of the cell (S.ivl) they come
        // within the support of (box distance per axis and half, summed
        // over the 8 combinations)
        {
            const uint32_t nst = S.nstaged;
            float lo[6], hi[6];
#pragma unroll
            for (int q = 0; q < 6; q++) {
                lo[q] = S.ivl[2 * q];
                hi[q] = S.ivl[2 * q + 1];
            }
            for (uint32_t k = tid; k < nst; k += NW * 32) {
                const float4 pc = S.r0[k];
                uint32_t m = 0u;
                if (pc.w != 0.f) {
                    const float x[3] = { pc.x, pc.y, pc.z };
                    float d2[6];
#pragma unroll
                    for (int q = 0; q < 6; q++) {
                        const float d = fmaxf(fmaxf(lo[q] - x[q >> 1], x[q >> 1] - hi[q]), 0.f);
                        d2[q] = d * d;
                    }
                    // (x half, y half) combinations, then z
                    const float dxy[4] = { d2[0] + d2[2], d2[1] + d2[2],
                                           d2[0] + d2[3], d2[1] + d2[3] };
#pragma unroll
                    for (int o = 0; o < 8; o++)
                        if (dxy[o & 3] + d2[4 + (o >> 2)] < R2)
                            m |= 1u << o;
                    if (pc.w < 0.f)
                        m <<= kMaskWallShift;
                }
                S.mask[k] = (uint16_t)m;
            }
            if (tid < 3)
                S.mask[nst + tid] = 0;  // read with the last records' group of 4
        }
        __syncthreads();
        return true;
    };

    // sorted index of staged slot k (probe path only)
    auto sorted_of = [&](uint32_t k) -> uint32_t {
        for (uint32_t i = 0; i < S.npieces; i++) {
            const uint4 pc = S.piece[i];
            if (k >= pc.x && k < pc.x + pc.z)
                return pc.y + (k - pc.x);
        }
        return 0u;
    };

    const uint32_t n_work = a.sc->n_chunks;
    // The next cell of the block (one thread decides for the block: another
    // block may set the error word at any time, and every thread must see
    // the same decision).  Thread 0 takes the next cell's index while the
    // current cell is swept; it reaches S.work before the cell's last
    // barrier.
    auto fetch = [&]() -> uint32_t {
        uint32_t w = a.sc->err ? 0xffffffffu : atomicAdd(&a.sc->chunk_next, 1u);
        // rate sample: skip the cells outside it
        while (c.sample_on && w < n_work) {
            const uint32_t k = a.b.work[w].x;
            if (sample_hash(k, c.sample_seed) < c.sample_thr || a.b.cell_mark[k])
                break;
            w = atomicAdd(&a.sc->chunk_next, 1u);
        }
        return w;
    };
    if (tid == 0)
        S.work = fetch();
    __syncthreads();
    uint32_t w_next = 0xffffffffu;  // thread 0
    for (;;) {
        const uint32_t w = S.work;
        if (w >= n_work)
            break;
        const uint4 wc = a.b.wcl[w];
        const uint32_t key = a.b.work[w].x;
        const uint32_t n_cl = wc.w;
        const uint32_t kc = wc.z;
        const CaseScalars& cas = a.cs[kc];
        const float dt = cas.dt;
        if (warp == 0 && lane < 9)
            S.row[lane] = a.b.crow[(size_t)w * 9 + lane];
        __syncthreads();
        if (tid == 0) {
            uint32_t t = 0;
            for (int r = 0; r < 9; r++)
                t += S.row[r].y;
            S.total = t;
        }
        __syncthreads();
        const uint32_t npass = (S.total + CAP - 1) / CAP;
        const bool single = npass <= 1;
        if (warp == NW - 1) {
            // the octant boxes of the cell: per axis and half, the extent of
            // the cell's particles that take neighbour sums (probes apart);
            // an empty half stays [+inf, -inf] and is never within reach.
            // Ready before the classification (stage's barrier).
            const float sc2 = 2.f * c.idist;
            float bl[6], bh[6];
#pragma unroll
            for (int q = 0; q < 6; q++) {
                bl[q] = INFINITY;
                bh[q] = -INFINITY;
            }
            for (uint32_t sidx = wc.x + lane; sidx < wc.y; sidx += 32) {
                const int imv = T.imove[sidx];
                if (imv < -3 || imv > 1 || imv == 0)
                    continue;
                const float4 p = a.b.rec0[sidx];
                const uint32_t o = cl_octant(p, cas, sc2);
                const float x[3] = { p.x, p.y, p.z };
#pragma unroll
                for (int ax = 0; ax < 3; ax++) {
                    // constant indices (registers): half 0 or 1 by select
                    const bool up = (o >> ax) & 1u;
                    bl[2 * ax] = up ? bl[2 * ax] : fminf(bl[2 * ax], x[ax]);
                    bh[2 * ax] = up ? bh[2 * ax] : fmaxf(bh[2 * ax], x[ax]);
                    bl[2 * ax + 1] = up ? fminf(bl[2 * ax + 1], x[ax]) : bl[2 * ax + 1];
                    bh[2 * ax + 1] = up ? fmaxf(bh[2 * ax + 1], x[ax]) : bh[2 * ax + 1];
                }
            }
#pragma unroll
            for (int q = 0; q < 6; q++) {
                for (int o = 16; o > 0; o >>= 1) {
                    bl[q] = fminf(bl[q], __shfl_xor_sync(0xffffffffu, bl[q], o));
                    bh[q] = fmaxf(bh[q], __shfl_xor_sync(0xffffffffu, bh[q], o));
                }
            }
            if (lane < 6) {
                float l = bl[0], h = bh[0];
#pragma unroll
                for (int q = 1; q < 6; q++)
                    if (lane == (uint32_t)q) {
                        l = bl[q];
                        h = bh[q];
                    }
                S.ivl[2 * lane] = l;
                S.ivl[2 * lane + 1] = h;
            }
        }
        bool failed = !stage(0);
        if (tid == 0)
            w_next = fetch();  // consumed at the end of this cell
        // single pass: each warp takes every NW-th cluster; several passes:
        // waves of NW clusters, each wave re-staging every pass
        const uint32_t waves = single ? 1u : (n_cl + NW - 1) / NW;
        for (uint32_t wave = 0; wave < waves && !failed; wave++) {
            const uint32_t c_begin = single ? (uint32_t)warp : wave * NW + warp;
            const uint32_t c_step = single ? (uint32_t)NW : 0xffffffffu;
            for (uint32_t ci = c_begin; ; ci += c_step) {
                const bool have = ci < n_cl;
                if (single && !have)
                    break;
                // ---- cluster set-up
                uint2 cl = make_uint2(0u, 0u);
                if (have)
                    cl = a.b.clu[wc.x + ci];
                const bool valid = (uint32_t)mq < cl.y;
                const uint32_t i = a.b.cperm[cl.x + (valid ? (uint32_t)mq : 0u)];
                const float4 r0i = a.b.rec0[i];
                const float4 r1i = a.b.rec1[i];
                const int im = T.imove[i];
                const bool want = valid && im >= -3 && im <= 1;
                const bool fluid = valid && im == 1;
                const bool sensor = valid && im == 0;
                const bool any_fluid = __any_sync(0xffffffffu, fluid);
                const bool probes = __any_sync(0xffffffffu, sensor);
                const bool any_want = __any_sync(0xffffffffu, want);
                // the octants of the cluster's particles that take sums: the
                // candidates are the staged records within the support of
                // any of those octant boxes (each box holds its particles,
                // so the list is conservative)
                const uint32_t omask = __reduce_or_sync(
                    0xffffffffu, want && !sensor ? 1u << cl_octant(r0i, cas, 2.f * c.idist) : 0u);
                float shep = 0.f, gp0 = 0.f, gp1 = 0.f, gp2 = 0.f;
                float lu0 = 0.f, lu1 = 0.f, lu2 = 0.f, du = 0.f, lp = 0.f;
                float gw0 = 0.f, gw1 = 0.f, gw2 = 0.f, dbi = 0.f;
                const float pi = r1i.w;
                uint32_t wfill = 0;
                bool walls_global = !single;
                uint16_t* list = S.list[warp];
                uint16_t* wl = S.wall[warp];

                // one fluid neighbour (staged records pj, vj) of this lane's
                // particle
                auto fluid_pair = [&](const float4 pj, const float4 vj) {
                    const float d0 = pj.x - r0i.x, d1 = pj.y - r0i.y, d2 = pj.z - r0i.z;
                    const float rr = d0 * d0 + d1 * d1 + d2 * d2;
                    const float rd = sqrtf(rr);
                    // (2 - q)^+ with q = rd / H: zero at and beyond the
                    // support (2)
                    const float tq = fmaxf(fmaf(-rd, c.inv_H, 2.f), 0.f);
                    const float tq2 = tq * tq;
                    // pj.w = CONW W-factor * m/rho: F(q) CONF m/rho up to
                    // the factor f_over_w, and W(q) CONW m/rho =
                    // (1 + 2q) (2 - q) gf, summed here as half of it,
                    // (1/2 + q) (2 - q) gf = (5/2 (2 - q) - (2 - q)^2) gf
                    // (zero with gf beyond the support; doubled once after
                    // the sums)
                    const float gf = tq2 * tq * pj.w;
                    shep = fmaf(fmaf(2.5f, tq, -tq2), gf, shep);
                    const float dv0 = vj.x - r1i.x, dv1 = vj.y - r1i.y, dv2 = vj.z - r1i.z;
                    const float udr = dv0 * d0 + dv1 * d1 + dv2 * d2;
                    const float t = (pi + vj.w) * gf;
                    gp0 = gp0 + t * d0;
                    gp1 = gp1 + t * d1;
                    gp2 = gp2 + t * d2;
                    lu0 = lu0 + gf * dv0;
                    lu1 = lu1 + gf * dv1;
                    lu2 = lu2 + gf * dv2;
                    du = du + udr * gf;
                    lp = lp + (vj.w - pi) * gf;
                };
                // one boundary element (staged records pj, nj): BIe wall sums
                auto wall_pair = [&](const float4 pj, const float4 nj) {
                    const float d0 = pj.x - r0i.x, d1 = pj.y - r0i.y, d2 = pj.z - r0i.z;
                    const float rr = d0 * d0 + d1 * d1 + d2 * d2;
                    const float qq = sqrtf(rr) * c.inv_H;
                    const float tq = fmaxf(2.f - qq, 0.f);
                    const float tq2 = tq * tq;
                    const float wa = c.w_conw * (1.f + 2.f * qq) * tq2 * tq2 * (-pj.w);
                    gw0 = gw0 + nj.x * wa;
                    gw1 = gw1 + nj.y * wa;
                    gw2 = gw2 + nj.z * wa;
                    dbi = dbi - nj.w * wa;
                };
                // sums the first nq quads of a list (lane takes slot q); the
                // load latency is left to the other resident warps (a
                // software prefetch of the next entry cost registers and
                // was slower)
                auto drain = [&](const uint16_t* lst, uint32_t nq, bool walls) {
                    if (nq == 0)
                        return;
                    for (uint32_t t = 0; t < nq; t++) {
                        const uint32_t j = lst[4 * t + q];
                        const float4 a0 = S.r0[j], a1 = S.r1[j];
                        if (walls)
                            wall_pair(a0, a1);
                        else
                            fluid_pair(a0, a1);
                    }
                };

                for (uint32_t p = 0; p < npass && !failed; p++) {
                    if (p > 0 || wave > 0) {  // pass 0 of wave 0 is staged
                        __syncthreads();
                        failed = !stage(p);
                        if (failed)
                            break;
                    }
                    if (!have || !any_want)
                        continue;
                    const uint32_t nst = S.nstaged;
                    if (probes) {
                        // probe cluster: lane m < 8 sums probe m over every
                        // staged record (cfd/Sensors.cl: fluid neighbours)
                        const uint32_t ip = a.b.cperm[cl.x + min((uint32_t)lane, cl.y - 1u)];
                        const float4 rp = a.b.rec0[ip];
                        float sh = 0.f, s0 = 0.f, s1 = 0.f, s2 = 0.f, sr = 0.f, sp = 0.f;
                        if ((uint32_t)lane < cl.y && T.imove[ip] == 0) {
                            for (uint32_t j = 0; j < nst; j++) {
                                const float4 pj = S.r0[j];
                                if (!(pj.w > 0.f))
                                    continue;
                                const float d0 = pj.x - rp.x, d1 = pj.y - rp.y, d2 = pj.z - rp.z;
                                const float qq = sqrtf(d0 * d0 + d1 * d1 + d2 * d2) * c.inv_H;
                                if (qq >= c.SUPPORT)
                                    continue;
                                const float4 vj = S.r1[j];
                                const float tq = 2.f - qq;
                                const float tq2 = tq * tq;
                                const float wq = (1.f + 2.f * qq) * tq2 * tq2;
                                const float wp = c.w_conw * wq;
                                const float wj = wq * pj.w;
                                sh = sh + wj;
                                s0 = s0 + vj.x * wj;
                                s1 = s1 + vj.y * wj;
                                s2 = s2 + vj.z * wj;
                                sr = sr + wp * T.m[sorted_of(j)];
                                sp = sp + vj.w * wj;
                            }
                        }
                        // into the quad layout: slot 0 of particle mq
                        const float v[6] = { sh, s0, s1, s2, sr, sp };
                        float o[6];
                        for (int k = 0; k < 6; k++) {
                            o[k] = __shfl_sync(0xffffffffu, v[k], mq);
                            if (q != 0)
                                o[k] = 0.f;
                        }
                        shep += 0.5f * o[0];  // doubled with the pair sums
                        gp0 += o[1];
                        gp1 += o[2];
                        gp2 += o[3];
                        du += o[4];
                        lp += o[5];
                        continue;
                    }
                    uint32_t fill = 0;
                    uint32_t wdone = wfill;  // wall entries already summed
                    // the boundary elements matter to fluid particles only
                    const uint32_t wmask = any_fluid ? omask << kMaskWallShift : 0u;
                    // 128 records per round, four per lane (records 4l ..
                    // 4l+3), listed in staging order
                    for (uint32_t base = 0; base < nst; base += 128) {
                        const uint32_t k0 = base + 4u * lane;
                        uint2 mm = make_uint2(0u, 0u);
                        if (k0 < nst)
                            mm = *reinterpret_cast<const uint2*>(&S.mask[k0]);
                        const uint32_t m[4] = { mm.x & 0xffffu, mm.x >> 16, mm.y & 0xffffu, mm.y >> 16 };
                        bool fl[4], wa[4];
                        unsigned bw[4];
                        uint32_t before = 0, wbefore = 0, tot = 0, wtot = 0;
#pragma unroll
                        for (int u = 0; u < 4; u++) {
                            fl[u] = (m[u] & omask) != 0u;
                            wa[u] = (m[u] & wmask) != 0u;
                            const unsigned bf = __ballot_sync(0xffffffffu, fl[u]);
                            bw[u] = __ballot_sync(0xffffffffu, wa[u]);
                            before += (uint32_t)__popc(bf & lt);
                            tot += (uint32_t)__popc(bf);
                            wtot |= bw[u];
                        }
                        {
                            uint32_t p = fill + before;
#pragma unroll
                            for (int u = 0; u < 4; u++)
                                if (fl[u])
                                    list[p++] = (uint16_t)(k0 + u);
                        }
                        fill += tot;
                        if (wtot) {
#pragma unroll
                            for (int u = 0; u < 4; u++)
                                wbefore += (uint32_t)__popc(bw[u] & lt);
                            wtot = 0;
#pragma unroll
                            for (int u = 0; u < 4; u++)
                                wtot += (uint32_t)__popc(bw[u]);
                            if (wfill + wtot > (uint32_t)kClWallCap) {
                                // the wall list is full: sum it, and let the
                                // epilogue walk the walls from global memory
                                __syncwarp();
                                const uint32_t n = wfill - wdone;
                                if (lane < (int)((4 - (n & 3)) & 3))
                                    wl[wfill + lane] = (uint16_t)CAP;
                                __syncwarp();
                                drain(wl + wdone, (n + 3) / 4, true);
                                __syncwarp();
                                wfill = 0;
                                wdone = 0;
                                walls_global = true;
                            }
                            uint32_t q = wfill + wbefore;
#pragma unroll
                            for (int u = 0; u < 4; u++)
                                if (wa[u])
                                    wl[q++] = (uint16_t)(k0 + u);
                            wfill += wtot;
                        }
                        if (fill > (uint32_t)(kClListCap - 128)) {
                            __syncwarp();
                            const uint32_t nq = fill / 4;
                            drain(list, nq, false);
                            __syncwarp();
                            const uint32_t rem = fill - 4 * nq;
                            uint16_t mv = 0;
                            if ((uint32_t)lane < rem)
                                mv = list[4 * nq + lane];
                            __syncwarp();
                            if ((uint32_t)lane < rem)
                                list[lane] = mv;
                            fill = rem;
                        }
                    }
                    // the rest of both lists, padded with the zero record
                    __syncwarp();
                    if ((uint32_t)lane < ((4u - (fill & 3u)) & 3u))
                        list[fill + lane] = (uint16_t)CAP;
                    const uint32_t nw_ = wfill - wdone;
                    if ((uint32_t)lane < ((4u - (nw_ & 3u)) & 3u))
                        wl[wfill + lane] = (uint16_t)CAP;
                    __syncwarp();
                    drain(list, (fill + 3) / 4, false);
                    drain(wl + wdone, (nw_ + 3) / 4, true);
                    __syncwarp();
                    if (!single)
                        wfill = 0;  // the staged records are replaced
                }
                if (failed)
                    break;
                if (have) {
                    shep = shep + shep;  // the pair sums hold half of it
                    // ---- the four partial sums of each particle
                    float* acc[13] = { &shep, &gp0, &gp1, &gp2, &lu0, &lu1, &lu2,
                                       &du, &lp, &gw0, &gw1, &gw2, &dbi };
#pragma unroll
                    for (int k = 0; k < 13; k++) {
                        float v = *acc[k];
                        v = v + __shfl_xor_sync(0xffffffffu, v, 8);
                        v = v + __shfl_xor_sync(0xffffffffu, v, 16);
                        *acc[k] = v;
                    }
                    const float v = sweep_cl_finish(
                        c, a, i, valid, im, want, fluid, sensor, q == 0, dt,
                        r0i, r1i, shep, gp0, gp1, gp2, lu0, lu1, lu2, du, lp,
                        gw0, gw1, gw2, dbi, walls_global, wl, wfill, S.r0,
                        S.r1, key, cas);
                    float vm = v;
                    for (int o = 16; o > 0; o >>= 1)
                        vm = cl_min(vm, __shfl_xor_sync(0xffffffffu, vm, o));
                    if (kc != run_case) {
                        flush();
                        run_case = kc;
                        run_min = INFINITY;
                    }
                    run_min = cl_min(run_min, vm);
                }
                if (!single)
                    break;  // one cluster per warp per wave
                __syncwarp();
            }
        }
        if (failed)
            break;
        if (tid == 0)
            S.work = w_next;  // every thread read this cell's S.work long ago
        __syncthreads();  // the staged records are rewritten for the next cell
    }
    flush();
}

}  // namespace
