/*
 * CPU oracle: a restatement of AQUAgpusph's per-step WCSPH pipeline (the
 * canonical preset stack basic + midpoint + domain + cfd + deltaSPH + BIe +
 * variableTimeStep, Morris viscosity, Wendland kernel).
 *
 * TEST INFRASTRUCTURE ONLY.  It is the oracle of the CUDA library and the
 * timed CPU baseline of bench.py; the product never links it.  It is pinned
 * by tests/test_oracle_pin.py against (a) the reference's own kernel sources
 * compiled on the host (oracle/refshim/ref_kernels.cpp, bit-exact on whole
 * steps) and (b) the golden fixtures and assertions of the reference's own
 * tests (tests/{2D,3D}/LinkList, tests/3D/RadixSort, tests/2D/Regressions).
 *
 * Floating point: IEEE binary32, every operation in the reference's source
 * order, no FMA contraction (-ffp-contract=off), divisions and square roots
 * correctly rounded.  Reductions of min/max are order independent.
 *
 * Source of each stage (paths relative to the reference tree):
 *   link-list ........ aquagpusph/CalcServer/LinkList.cpp:185-232, 326-494;
 *                      LinkList.cl.in:32-113
 *   radix sort ....... aquagpusph/CalcServer/RadixSort.cpp:130-304 (stable)
 *   predictor etc. ... resources/Scripts/basic/time_scheme/midpoint.cl:53-227
 *   Domain ........... resources/Scripts/basic/Domain.cl:48-90
 *   sort stage1/2 .... resources/Scripts/basic/Sort.cl:57-124
 *   EOS, Binormal .... resources/Scripts/basic/EOS.cl:57-73, Binormal.cl:37-53
 *   Wendland ......... resources/Scripts/KernelFunctions/Wendland{2D,3D}.hcl:44-66
 *   neighbour order .. resources/Scripts/types/{2D.h:174-194,3D.h:197-219}
 *   Shepard .......... resources/Scripts/basic/Shepard.cl:76-125 (cfd/Shepard.cl)
 *   interactions ..... resources/Scripts/cfd/Interactions.cl:60-145
 *   sensors .......... resources/Scripts/cfd/Sensors.cl:57-130,
 *                      cfd/SensorsRenormalization.cl:42-67
 *   delta-SPH ........ resources/Scripts/basic/deltaSPH.cl:191-242, 330-350
 *   BIe .............. resources/Scripts/cfd/Boundary/BIe/Interactions.cl:48-108,
 *                      Rates.cl:44-62, ElasticBounce.cl:64-152, PST.cl:62-110
 *   rates ............ resources/Scripts/cfd/Rates.cl:55-77
 *   time step ........ resources/Scripts/cfd/TimeStep.cl:56-77,
 *                      Presets/src/cfd/variableTimeStep.xml:11-16
 */
#include "aqua_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>
#include <omp.h>

namespace {

/* -------------------------------------------------------------- helpers */

/* OpenCL min/max semantics for floats */
inline float fmin_cl(float x, float y) { return (y < x) ? y : x; }
inline float fmax_cl(float x, float y) { return (x < y) ? y : x; }

template<typename F>
void
par_for(uint32_t n, int nt, F&& f)
{
#pragma omp parallel for schedule(static) num_threads(nt)
    for (long i = 0; i < (long)n; i++)
        f((uint32_t)i);
}

/* Wendland C2 kernel, q = |r_ij| / h, support 2 (Wendland{2D,3D}.hcl:44-66).
 * The constant factors are float products folded at compile time, as the
 * OpenCL compiler folds them. */
template<int D>
struct Wendland;
template<>
struct Wendland<3>
{
    static constexpr float wconW = 0.08203125f * 0.318309886f;
    static constexpr float wconF = 0.8203125f * 0.318309886f;
};
template<>
struct Wendland<2>
{
    static constexpr float wconW = 0.109375f * 0.318309886f;
    static constexpr float wconF = 1.09375f * 0.318309886f;
};
template<int D>
inline float
kernel_w(float q)
{
    const float a = 2.f - q;
    float w = Wendland<D>::wconW * (1.f + 2.f * q);
    w = w * a;
    w = w * a;
    w = w * a;
    return w * a;
}
template<int D>
inline float
kernel_f(float q)
{
    const float a = 2.f - q;
    float f = Wendland<D>::wconF * a;
    f = f * a;
    return f * a;
}

/* Vectors of the reference layout: VS floats per particle, of which the
 * first D are the spatial components (the `.XYZ` part). */
template<int D>
struct V
{
    static constexpr int VS = (D == 3) ? 4 : 2;
    float c[VS];
};

template<int D>
inline float
dot_xyz(const float* a, const float* b)
{
    float s = a[0] * b[0];
    for (int k = 1; k < D; k++)
        s = s + a[k] * b[k];
    return s;
}
/* dot over the full storage vector (float4 in 3-D, incl. w) */
template<int D>
inline float
dot_full(const float* a, const float* b)
{
    float s = a[0] * b[0];
    for (int k = 1; k < V<D>::VS; k++)
        s = s + a[k] * b[k];
    return s;
}

/* The state and parameters of one case, with the per-case Definitions */
template<int D>
struct Case
{
    static constexpr int VS = V<D>::VS;
    aq_state* st;
    const aq_params* pr;
    int nt;
    uint32_t N;

    float* vec(float* p, uint32_t i) const { return p + (size_t)VS * i; }
    const float* vec(const float* p, uint32_t i) const { return p + (size_t)VS * i; }
};

/* --------------------------------------------------------- link-list */

/* Neighbour cells of c_i in the reference visiting order (x offset
 * outermost, z innermost); returns their number. */
template<int D>
inline int
neighbour_cells(uint32_t c_i, const uint32_t* n_cells, uint32_t* out)
{
    int k = 0;
    if (D == 3) {
        const uint32_t nx = n_cells[0], nxy = n_cells[0] * n_cells[1];
        for (int ci = -1; ci <= 1; ci++)
            for (int cj = -1; cj <= 1; cj++)
                for (int ck = -1; ck <= 1; ck++)
                    out[k++] = c_i + (uint32_t)ci + (uint32_t)cj * nx +
                               (uint32_t)ck * nxy;
    } else {
        const uint32_t nx = n_cells[0];
        for (int ci = -1; ci <= 1; ci++)
            for (int cj = -1; cj <= 1; cj++)
                out[k++] = c_i + (uint32_t)ci + (uint32_t)cj * nx;
    }
    return k;
}

/* Visit every particle j of the neighbour cells of particle i, in the
 * reference order; f(j) is called for each (filters are up to f). */
template<int D, typename F>
inline void
for_neighbours(const aq_state* st, uint32_t i, F&& f)
{
    uint32_t cells[27];
    const int nc = neighbour_cells<D>(st->icell[i], st->n_cells, cells);
    const uint32_t N = st->N;
    for (int k = 0; k < nc; k++) {
        const uint32_t c = cells[k];
        for (uint32_t j = st->ihoc[c]; j < N && st->icell[j] == c; j++)
            f(j);
    }
}

template<int D>
int
linklist(Case<D>& cs)
{
    aq_state* st = cs.st;
    const aq_params* pr = cs.pr;
    const uint32_t N = cs.N;
    const int VS = Case<D>::VS;

    /* r_min / r_max of r_in over all N (Reduction tools, identities
     * +-VEC_INFINITY whose w is 0) */
    float mn[4] = { INFINITY, INFINITY, INFINITY, 0.f };
    float mx[4] = { -INFINITY, -INFINITY, -INFINITY, -0.f };
    if (D == 2) {
        mn[2] = mn[3] = mx[2] = mx[3] = 0.f;
    }
    for (uint32_t i = 0; i < N; i++) {
        const float* r = cs.vec(st->r_in, i);
        for (int k = 0; k < VS; k++) {
            mn[k] = fmin_cl(mn[k], r[k]);
            mx[k] = fmax_cl(mx[k], r[k]);
        }
    }
    std::memcpy(st->r_min, mn, sizeof(mn));
    std::memcpy(st->r_max, mx, sizeof(mx));

    /* n_cells: (max - min) / (support*h) in float, truncated, + 6 */
    const float cell_length = pr->support * pr->h;
    if (!(cell_length > 0.f))
        return AQ_ERR_INVALID;
    uint64_t n[3] = { 1, 1, 1 };
    for (int k = 0; k < D; k++) {
        const float span = (mx[k] - mn[k]) / cell_length;
        if (!(span >= 0.f) || span > 4.0e9f)
            return AQ_ERR_INVALID;
        n[k] = (uint64_t)span + 6;
    }
    const uint64_t nw = n[0] * n[1] * n[2];
    if (nw > st->ihoc_capacity || nw > 0xffffffffull)
        return AQ_ERR_CAPACITY;
    st->n_cells[0] = (uint32_t)n[0];
    st->n_cells[1] = (uint32_t)n[1];
    st->n_cells[2] = (uint32_t)n[2];
    st->n_cells[3] = (uint32_t)nw;

    /* icell: (r - r_min) * (1 / (support*h)), truncated, + 2 per axis */
    const float idist = 1.f / (pr->support * pr->h);
    par_for(N, cs.nt, [&](uint32_t i) {
        const float* r = cs.vec(st->r_in, i);
        uint32_t a[3] = { 0, 0, 0 };
        for (int k = 0; k < D; k++)
            a[k] = (uint32_t)(uint64_t)((r[k] - mn[k]) * idist) + 2u;
        uint32_t c = a[0] + a[1] * st->n_cells[0];
        if (D == 3)
            c += a[2] * st->n_cells[0] * st->n_cells[1];
        st->icell[i] = c;
    });

    /* stable sort of icell in the current order */
    aq_sort(st->icell, st->id_unsorted, st->id_sorted, N);

    /* ihoc: N for empty cells, first sorted index otherwise */
    std::fill(st->ihoc, st->ihoc + nw, N);
    for (uint32_t i = N; i-- > 0;)
        st->ihoc[st->icell[i]] = i;
    return AQ_OK;
}

/* ------------------------------------------------------ prescribed roll */

/* Rolls the boundary elements and probes of the roll set from the angle at
 * t_before to the angle at t_after about z through roll_center: the
 * reference's motion tools UnTransform (previous angle), Velocity and
 * Transform (new angle), cfd/Motions/{UnTransform,Velocity,Transform}.cl.
 * Angles, rate, cosines and sines are evaluated in double and rounded. */
template<int D>
void
roll(Case<D>& cs, float t_before, float t_after)
{
    aq_state* st = cs.st;
    const aq_params* pr = cs.pr;
    const int VS = Case<D>::VS;
    const double w = pr->roll_angular_freq, A = pr->roll_amplitude;
    const float psi_in = (float)(A * std::sin(w * (double)t_before));
    const float psi = (float)(A * std::sin(w * (double)t_after));
    const float omega = (float)(A * w * std::cos(w * (double)t_after));
    const float ci = (float)std::cos((double)psi_in);
    const float si = -(float)std::sin((double)psi_in);
    const float cp = (float)std::cos((double)psi);
    const float sp = (float)std::sin((double)psi);
    par_for(cs.N, cs.nt, [&](uint32_t i) {
        if (st->iset[i] != pr->roll_iset || st->imove[i] == 1)
            return;
        float* r = cs.vec(st->r, i);
        float* n = cs.vec(st->normal, i);
        float* t = cs.vec(st->tangent, i);
        float* u = cs.vec(st->u, i);
        float rr[4] = { 0.f, 0.f, 0.f, 0.f };
        for (int d = 0; d < VS; d++)
            rr[d] = r[d] - pr->roll_center[d];
        float rl[4], nl[4], tl[4];
        for (int d = 0; d < 4; d++) {
            rl[d] = d < VS ? rr[d] : 0.f;
            nl[d] = d < VS ? n[d] : 0.f;
            tl[d] = d < VS ? t[d] : 0.f;
        }
        rl[0] = ci * rr[0] - si * rr[1];
        rl[1] = si * rr[0] + ci * rr[1];
        nl[0] = ci * n[0] - si * n[1];
        nl[1] = si * n[0] + ci * n[1];
        tl[0] = ci * t[0] - si * t[1];
        tl[1] = si * t[0] + ci * t[1];
        const float ul0 = -omega * rl[1], ul1 = omega * rl[0];
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
        float nn = 0.f, tt = 0.f;
        for (int d = 0; d < VS; d++) {
            ro[d] = ro[d] + pr->roll_center[d];
            nn = nn + no[d] * no[d];
            tt = tt + to[d] * to[d];
        }
        nn = std::sqrt(nn);
        tt = std::sqrt(tt);
        for (int d = 0; d < VS; d++) {
            r[d] = ro[d];
            n[d] = no[d] / nn;
            t[d] = to[d] / tt;
            u[d] = 0.f;
        }
        u[0] = cp * ul0 - sp * ul1;
        u[1] = sp * ul0 + cp * ul1;
    });
}

/* --------------------------------------------------------- one step */

template<int D>
int
step(Case<D>& cs)
{
    aq_state* st = cs.st;
    const aq_params* pr = cs.pr;
    const uint32_t N = cs.N;
    const int VS = Case<D>::VS;
    const int nt = cs.nt;
    const float dt = st->dt;
    const float H = pr->H, CONW = pr->CONW, CONF = pr->CONF;
    const float SUPPORT = pr->SUPPORT;

    /* predictor: back up r, u, dudt, rho, drhodt; then Domain on the
     * backups (out-of-domain or non-finite -> buffer particle) */
    par_for(N, nt, [&](uint32_t i) {
        std::memcpy(cs.vec(st->r_in, i), cs.vec(st->r, i), VS * sizeof(float));
        std::memcpy(cs.vec(st->u_in, i), cs.vec(st->u, i), VS * sizeof(float));
        std::memcpy(cs.vec(st->dudt_in, i), cs.vec(st->dudt, i), VS * sizeof(float));
        st->rho_in[i] = st->rho[i];
        st->drhodt_in[i] = st->drhodt[i];
        if (st->imove[i] <= -255)
            return;
        const float* x = cs.vec(st->r_in, i);
        bool out = false;
        for (int k = 0; k < D; k++)
            out = out || std::isnan(x[k]) || std::isinf(x[k]) ||
                  x[k] < pr->domain_min[k] || x[k] > pr->domain_max[k];
        if (out) {
            st->imove[i] = -256;
            st->m[i] = 0.f;
            std::memset(cs.vec(st->u_in, i), 0, VS * sizeof(float));
            std::memset(cs.vec(st->dudt_in, i), 0, VS * sizeof(float));
            std::memcpy(cs.vec(st->r_in, i), pr->domain_max, VS * sizeof(float));
        }
    });

    int err = linklist<D>(cs);
    if (err)
        return err;

    /* backups of the sorted-by-copy fields, then the two sort stages:
     * new[id_sorted[i]] = old[i]; the old rates go to dudt_in/drhodt_in */
    std::memcpy(st->id_in, st->id, N * sizeof(uint32_t));
    std::memcpy(st->iset_in, st->iset, N * sizeof(uint32_t));
    std::memcpy(st->imove_in, st->imove, N * sizeof(int32_t));
    std::memcpy(st->normal_in, st->normal, (size_t)N * VS * sizeof(float));
    std::memcpy(st->tangent_in, st->tangent, (size_t)N * VS * sizeof(float));
    std::memcpy(st->m_in, st->m, N * sizeof(float));
    par_for(N, nt, [&](uint32_t i) {
        const uint32_t o = st->id_sorted[i];
        st->id[o] = st->id_in[i];
        st->iset[o] = st->iset_in[i];
        st->imove[o] = st->imove_in[i];
        std::memcpy(cs.vec(st->r, o), cs.vec(st->r_in, i), VS * sizeof(float));
        std::memcpy(cs.vec(st->normal, o), cs.vec(st->normal_in, i), VS * sizeof(float));
        std::memcpy(cs.vec(st->tangent, o), cs.vec(st->tangent_in, i), VS * sizeof(float));
    });
    par_for(N, nt, [&](uint32_t i) {
        const uint32_t o = st->id_sorted[i];
        st->rho[o] = st->rho_in[i];
        st->m[o] = st->m_in[i];
        std::memcpy(cs.vec(st->u, o), cs.vec(st->u_in, i), VS * sizeof(float));
        std::memcpy(cs.vec(st->dudt_in, o), cs.vec(st->dudt, i), VS * sizeof(float));
        st->drhodt_in[o] = st->drhodt[i];
    });

    /* linear EOS on fluid/solid (imove > 0) and fixed (imove == -1)
     * particles; Binormal */
    auto eos = [&](uint32_t i) {
        const int im = st->imove[i];
        if (im <= 0 && im != -1)
            return;
        st->p[i] = pr->p0 + pr->cs * pr->cs * (st->rho[i] - pr->refd[st->iset[i]]);
    };
    par_for(N, nt, eos);
    par_for(N, nt, [&](uint32_t i) {
        float* b = cs.vec(st->binormal, i);
        const float* nn = cs.vec(st->normal, i);
        float* t = cs.vec(st->tangent, i);
        if (D == 3) {
            b[0] = nn[1] * t[2] - nn[2] * t[1];
            b[1] = nn[2] * t[0] - nn[0] * t[2];
            b[2] = nn[0] * t[1] - nn[1] * t[0];
            b[3] = 0.f;
        } else {
            b[0] = 0.f;
            b[1] = 0.f;
            t[0] = nn[1];
            t[1] = -nn[0];
        }
    });

    /* midpoint loop set-up: copies, then iterations */
    std::memcpy(st->drhodt, st->drhodt_in, N * sizeof(float));
    std::memcpy(st->dudt, st->dudt_in, (size_t)N * VS * sizeof(float));
    std::memcpy(st->r_in, st->r, (size_t)N * VS * sizeof(float));
    std::memcpy(st->u_in, st->u, (size_t)N * VS * sizeof(float));
    std::memcpy(st->rho_in, st->rho, N * sizeof(float));
    std::fill(st->lap_p, st->lap_p + N, 0.f);
    std::fill(st->lap_u, st->lap_u + (size_t)N * VS, 0.f);
    std::fill(st->div_u, st->div_u + N, 0.f);
    std::fill(st->grad_p, st->grad_p + (size_t)N * VS, 0.f);
    std::fill(st->shepard, st->shepard + N, 0.f);

    const float half_dt = 0.5f * dt;
    for (uint32_t it = 0; it < pr->iter_midpoint_max; it++) {
        std::memcpy(st->drhodt_in, st->drhodt, N * sizeof(float));
        std::memcpy(st->dudt_in, st->dudt, (size_t)N * VS * sizeof(float));
        /* half step, EOS */
        par_for(N, nt, [&](uint32_t i) {
            if (st->imove[i] <= 0)
                return;
            const float* ui = cs.vec(st->u_in, i);
            const float* a = cs.vec(st->dudt, i);
            float* u = cs.vec(st->u, i);
            for (int k = 0; k < VS; k++)
                u[k] = ui[k] + half_dt * a[k];
            st->rho[i] = st->rho_in[i] + half_dt * st->drhodt[i];
        });
        par_for(N, nt, eos);

        /* Shepard: i in {-3..1} (fluid only among i > 0), over fluid j,
         * self included */
        par_for(N, nt, [&](uint32_t i) {
            const int im = st->imove[i];
            if (im < -3 || im > 1)
                return;
            const float* ri = cs.vec(st->r, i);
            float s = 0.f;
            for_neighbours<D>(st, i, [&](uint32_t j) {
                if (st->imove[j] != 1)
                    return;
                float d[3];
                const float* rj = cs.vec(st->r, j);
                for (int k = 0; k < D; k++)
                    d[k] = rj[k] - ri[k];
                const float q = std::sqrt(dot_xyz<D>(d, d)) / H;
                if (q >= SUPPORT)
                    return;
                s = s + kernel_w<D>(q) * CONW * st->m[j] / st->rho[j];
            });
            st->shepard[i] = s;
        });

        /* fluid-fluid interactions: grad p, Morris lap u, div u */
        par_for(N, nt, [&](uint32_t i) {
            if (st->imove[i] != 1)
                return;
            const float* ri = cs.vec(st->r, i);
            const float* ui = cs.vec(st->u, i);
            const float p_i = st->p[i], rho_i = st->rho[i];
            float gp[3] = { 0.f, 0.f, 0.f }, lu[3] = { 0.f, 0.f, 0.f }, du = 0.f;
            for_neighbours<D>(st, i, [&](uint32_t j) {
                if (j == i || st->imove[j] != 1)
                    return;
                const float* rj = cs.vec(st->r, j);
                const float* uj = cs.vec(st->u, j);
                float d[3], dv[3];
                for (int k = 0; k < D; k++)
                    d[k] = rj[k] - ri[k];
                const float q = std::sqrt(dot_xyz<D>(d, d)) / H;
                if (q >= SUPPORT)
                    return;
                const float rho_j = st->rho[j], p_j = st->p[j];
                for (int k = 0; k < D; k++)
                    dv[k] = uj[k] - ui[k];
                const float udr = dot_xyz<D>(dv, d);
                const float f_ij = kernel_f<D>(q) * CONF * st->m[j];
                const float sp = (p_i + p_j) / (rho_i * rho_j) * f_ij;
                const float sl = f_ij * 2.f / (rho_i * rho_j);
                for (int k = 0; k < D; k++) {
                    gp[k] = gp[k] + sp * d[k];
                    lu[k] = lu[k] + sl * dv[k];
                }
                du = du + udr * f_ij * rho_i / rho_j;
            });
            float* g = cs.vec(st->grad_p, i);
            float* l = cs.vec(st->lap_u, i);
            for (int k = 0; k < D; k++) {
                g[k] = gp[k];
                l[k] = lu[k];
            }
            st->div_u[i] = du;
        });

        /* sensors (imove == 0): Shepard-weighted fluid interpolation of u,
         * rho, p, then division by the Shepard factor (floor 1e-6 -> 1) */
        par_for(N, nt, [&](uint32_t i) {
            if (st->imove[i] != 0)
                return;
            const float* ri = cs.vec(st->r, i);
            float su[3] = { 0.f, 0.f, 0.f }, sr = 0.f, sp = 0.f;
            for_neighbours<D>(st, i, [&](uint32_t j) {
                if (j == i || st->imove[j] != 1)
                    return;
                const float* rj = cs.vec(st->r, j);
                float d[3];
                for (int k = 0; k < D; k++)
                    d[k] = rj[k] - ri[k];
                const float q = std::sqrt(dot_xyz<D>(d, d)) / H;
                if (q >= SUPPORT)
                    return;
                const float rho_j = st->rho[j];
                const float w = kernel_w<D>(q) * CONW * st->m[j] / rho_j;
                const float* uj = cs.vec(st->u, j);
                for (int k = 0; k < D; k++)
                    su[k] = su[k] + uj[k] * w;
                sr = sr + rho_j * w;
                sp = sp + st->p[j] * w;
            });
            float shep = st->shepard[i];
            if (shep < 1.0e-6f)
                shep = 1.f;
            float* u = cs.vec(st->u, i);
            for (int k = 0; k < D; k++)
                u[k] = su[k];
            for (int k = 0; k < VS; k++)
                u[k] = u[k] / shep;
            st->rho[i] = sr / shep;
            st->p[i] = sp / shep;
        });

        /* delta-SPH pressure Laplacian over fluid j != i */
        par_for(N, nt, [&](uint32_t i) {
            if (st->imove[i] != 1)
                return;
            const float* ri = cs.vec(st->r, i);
            const float p_i = st->p[i];
            float lp = 0.f;
            for_neighbours<D>(st, i, [&](uint32_t j) {
                if (j == i || st->imove[j] != 1)
                    return;
                const float* rj = cs.vec(st->r, j);
                float d[3];
                for (int k = 0; k < D; k++)
                    d[k] = rj[k] - ri[k];
                const float q = std::sqrt(dot_xyz<D>(d, d)) / H;
                if (q >= SUPPORT)
                    return;
                const float f = kernel_f<D>(q) * CONF * st->m[j] / st->rho[j];
                lp = lp + (st->p[j] - p_i) * f;
            });
            st->lap_p[i] = lp;
        });

        /* BIe wall sums over wall elements (imove == -3) */
        par_for(N, nt, [&](uint32_t i) {
            float* gw = cs.vec(st->grad_w_bi, i);
            for (int k = 0; k < VS; k++)
                gw[k] = 0.f;
            st->div_u_bi[i] = 0.f;
            if (st->imove[i] != 1)
                return;
            const float* ri = cs.vec(st->r, i);
            float g[3] = { 0.f, 0.f, 0.f }, dbi = 0.f;
            for_neighbours<D>(st, i, [&](uint32_t j) {
                if (st->imove[j] != -3)
                    return;
                const float* rj = cs.vec(st->r, j);
                float d[3];
                for (int k = 0; k < D; k++)
                    d[k] = rj[k] - ri[k];
                const float q = std::sqrt(dot_xyz<D>(d, d)) / H;
                if (q >= SUPPORT)
                    return;
                const float* nj = cs.vec(st->normal, j);
                const float* uj = cs.vec(st->u, j);
                const float wa = kernel_w<D>(q) * CONW * st->m[j];
                float gwj[3];
                for (int k = 0; k < D; k++) {
                    gwj[k] = nj[k] * wa;
                    g[k] = g[k] + gwj[k];
                }
                dbi = dbi - dot_xyz<D>(uj, gwj);
            });
            for (int k = 0; k < D; k++)
                gw[k] = g[k];
            st->div_u_bi[i] = dbi;
        });

        /* BIe rates, cfd rates, delta-SPH term (fluid only) */
        par_for(N, nt, [&](uint32_t i) {
            if (st->imove[i] != 1)
                return;
            const float rho_i = st->rho[i];
            const float* gw = cs.vec(st->grad_w_bi, i);
            const float* u = cs.vec(st->u, i);
            float* gp = cs.vec(st->grad_p, i);
            const float s = 2.f * st->p[i] / rho_i;
            for (int k = 0; k < VS; k++)
                gp[k] = gp[k] + s * gw[k];
            st->div_u[i] = st->div_u[i] -
                           2.f * rho_i * (dot_full<D>(u, gw) + st->div_u_bi[i]);
            const uint32_t set = st->iset[i];
            const float* lu = cs.vec(st->lap_u, i);
            float* a = cs.vec(st->dudt, i);
            const float visc = pr->visc_dyn[set];
            for (int k = 0; k < VS; k++)
                a[k] = -gp[k] + visc * lu[k] + pr->g[k];
            st->drhodt[i] = -st->div_u[i];
            const float delta_f = pr->delta[set] * dt * rho_i / pr->refd[set];
            st->drhodt[i] = st->drhodt[i] + delta_f * st->lap_p[i];
        });

        /* BIe elastic bounce: reflect the velocity against wall elements the
         * particle reaches within this step */
        if (dt != 0.f) {
            const float dr_factor = pr->dr_factor;
            const float mbd = pr->min_bound_dist;
            par_for(N, nt, [&](uint32_t i) {
                if (st->imove[i] != 1)
                    return;
                const float* ri = cs.vec(st->r_in, i);
                const float* uin = cs.vec(st->u_in, i);
                float* a = cs.vec(st->dudt, i);
                float acc[3], vh[3];
                for (int k = 0; k < D; k++) {
                    acc[k] = a[k];
                    vh[k] = uin[k] + half_dt * acc[k];
                }
                for_neighbours<D>(st, i, [&](uint32_t j) {
                    if (st->imove[j] != -3)
                        return;
                    const float* rj = cs.vec(st->r_in, j);
                    const float* nj = cs.vec(st->normal, j);
                    float d[3], t[3];
                    for (int k = 0; k < D; k++)
                        d[k] = rj[k] - ri[k];
                    const float rn = dot_xyz<D>(d, nj);
                    if (rn < 0.f)
                        return;
                    const float dr = (D == 3) ? std::sqrt(st->m[j]) : st->m[j];
                    const float R = dr_factor * dr;
                    for (int k = 0; k < D; k++)
                        t[k] = d[k] - rn * nj[k];
                    if (dot_xyz<D>(t, t) >= R * R)
                        return;
                    const float drn = dt * dot_xyz<D>(vh, nj);
                    if (drn < 0.f)
                        return;
                    if (rn - drn <= mbd * dr) {
                        float v[3], vr[3];
                        for (int k = 0; k < D; k++)
                            v[k] = uin[k] + dt * acc[k];
                        const float vn2 = 2.f * dot_xyz<D>(v, nj);
                        for (int k = 0; k < D; k++)
                            vr[k] = v[k] - vn2 * nj[k];
                        for (int k = 0; k < D; k++) {
                            acc[k] = (vr[k] - uin[k]) / dt;
                            vh[k] = uin[k] + half_dt * acc[k];
                        }
                    }
                });
                for (int k = 0; k < D; k++)
                    a[k] = acc[k];
            });
        }

        /* relax */
        const float rl = pr->relax_midpoint;
        par_for(N, nt, [&](uint32_t i) {
            if (st->imove[i] <= 0)
                return;
            const float* ai = cs.vec(st->dudt_in, i);
            float* a = cs.vec(st->dudt, i);
            for (int k = 0; k < VS; k++)
                a[k] = rl * ai[k] + (1.f - rl) * a[k];
            st->drhodt[i] = rl * st->drhodt_in[i] + (1.f - rl) * st->drhodt[i];
        });
    }

    /* corrector, then PST against the wall elements of the cell list */
    const float hdt2 = 0.5f * dt * dt;
    par_for(N, nt, [&](uint32_t i) {
        if (st->imove[i] <= 0)
            return;
        const float* ri = cs.vec(st->r_in, i);
        const float* ui = cs.vec(st->u_in, i);
        const float* a = cs.vec(st->dudt, i);
        float* r = cs.vec(st->r, i);
        float* u = cs.vec(st->u, i);
        for (int k = 0; k < VS; k++) {
            r[k] = ri[k] + dt * ui[k] + hdt2 * a[k];
            u[k] = ui[k] + dt * a[k];
        }
        st->rho[i] = st->rho_in[i] + dt * st->drhodt[i];
    });
    const float inv_dims = 1.f / pr->DIMS;
    par_for(N, nt, [&](uint32_t i) {
        if (st->imove[i] != 1)
            return;
        const float Ri = 0.5f * std::pow(st->m[i] / st->rho[i], inv_dims);
        float* r = cs.vec(st->r, i);
        for_neighbours<D>(st, i, [&](uint32_t j) {
            if (st->imove[j] != -3)
                return;
            const float* rj = cs.vec(st->r, j);
            const float* nj = cs.vec(st->normal, j);
            float d[3], t[3];
            for (int k = 0; k < D; k++)
                d[k] = rj[k] - r[k];
            const float rn = dot_xyz<D>(d, nj);
            if (std::fabs(rn) > Ri)
                return;
            const float dr = (D == 3) ? std::sqrt(st->m[j]) : st->m[j];
            const float Rj = pr->dr_factor * dr;
            for (int k = 0; k < D; k++)
                t[k] = d[k] - rn * nj[k];
            if (dot_xyz<D>(t, t) >= Rj * Rj)
                return;
            const float s = rn - Ri;
            for (int k = 0; k < D; k++)
                r[k] = r[k] + s * nj[k];
        });
    });

    /* variable time step and its minimum */
    const float dt_fixed = pr->dt_fixed;
    par_for(N, nt, [&](uint32_t i) {
        if (st->imove[i] <= 0) {
            st->dt_var[i] = dt_fixed;
            return;
        }
        const float* u = cs.vec(st->u, i);
        const float dr_max = pr->dt_Ma * pr->h;
        const float dt_u = pr->courant * dr_max / std::sqrt(dot_full<D>(u, u));
        st->dt_var[i] = fmax_cl(fmin_cl(dt_fixed, dt_u), pr->dt_min);
    });
    float dt_new = INFINITY;
    for (uint32_t i = 0; i < N; i++)
        dt_new = fmin_cl(dt_new, st->dt_var[i]);
    if (!(dt_new > 0.f))
        return AQ_ERR_DT;
    st->dt = dt_new;
    const float t_before = st->t;
    st->t = (float)((double)st->t + (double)dt_new);
    st->iter += 1;
    if (pr->roll_enabled)
        roll<D>(cs, t_before, st->t);
    return AQ_OK;
}

int
threads(int nthreads)
{
    return nthreads > 0 ? nthreads : omp_get_max_threads();
}

} // namespace

extern "C" int
aq_sort(uint32_t* keys, uint32_t* perm, uint32_t* inv_perm, uint32_t n)
{
    /* counting sort (stable): offsets by key, then placement in order */
    if (!n)
        return AQ_OK;
    const uint32_t kmax = *std::max_element(keys, keys + n);
    std::vector<uint32_t> off((size_t)kmax + 2, 0);
    for (uint32_t i = 0; i < n; i++)
        off[(size_t)keys[i] + 1]++;
    for (size_t k = 1; k < off.size(); k++)
        off[k] += off[k - 1];
    std::vector<uint32_t> sorted(n);
    for (uint32_t i = 0; i < n; i++) {
        const uint32_t s = off[keys[i]]++;
        sorted[s] = keys[i];
        perm[s] = i;
        inv_perm[i] = s;
    }
    std::memcpy(keys, sorted.data(), (size_t)n * sizeof(uint32_t));
    return AQ_OK;
}

extern "C" int
aq_linklist(aq_state* st, const aq_params* pr, int nthreads)
{
    if (!st || !pr || !st->N)
        return AQ_ERR_INVALID;
    if (pr->dims == 3) {
        Case<3> cs{ st, pr, threads(nthreads), st->N };
        return linklist<3>(cs);
    }
    if (pr->dims == 2) {
        Case<2> cs{ st, pr, threads(nthreads), st->N };
        return linklist<2>(cs);
    }
    return AQ_ERR_INVALID;
}

extern "C" int
aq_step(aq_state* st, const aq_params* pr, int nthreads)
{
    if (!st || !pr || !st->N)
        return AQ_ERR_INVALID;
    /* BI walls and the improved Euler scheme: only the reference-kernel
     * harness */
    if (pr->boundary != 0 || pr->scheme != 0)
        return AQ_ERR_INVALID;
    if (pr->dims == 3) {
        Case<3> cs{ st, pr, threads(nthreads), st->N };
        return step<3>(cs);
    }
    if (pr->dims == 2) {
        Case<2> cs{ st, pr, threads(nthreads), st->N };
        return step<2>(cs);
    }
    return AQ_ERR_INVALID;
}
