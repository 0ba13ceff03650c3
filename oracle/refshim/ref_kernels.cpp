/*
 * Reference-kernel harness.  TEST INFRASTRUCTURE ONLY -- never linked by the
 * product; built by oracle/Makefile into oracle/_ref/ where the reference
 * tree is present, and used by the CPU tests to pin the restatement in
 * oracle/aqua_oracle.cpp.
 *
 * The OpenCL kernel files of the reference's canonical WCSPH step are
 * #included unmodified (from the reference tree, via -I) into one namespace
 * each, on top of the OpenCL-C -> C++ shim in
 * oracle/refshim/resources/Scripts/types/types.h.  This file adds the host
 * side that the reference keeps in C++ (which needs OpenCL to build and so
 * cannot be compiled here), restated:
 *   - the preset tool order of one step, basic.xml:132-171 as modified by
 *     basic/time_scheme/midpoint.xml, basic/domain.xml, cfd.xml,
 *     cfd/deltaSPH.xml, cfd/BIe.xml and cfd/variableTimeStep.xml, or with
 *     cfd/BI.xml in place of cfd/BIe.xml (boundary = 1), and with
 *     basic/time_scheme/improved_euler.xml in place of the midpoint scheme
 *     (scheme = 1);
 *   - the link-list host logic, LinkList.cpp:185-232 (n_cells, float
 *     division by support*h) and LinkList.cpp:326-494 (tool sequence);
 *   - the radix-sort tool as the stable sort it is (RadixSort.cpp:130-304,
 *     LSD passes of RadixSort.cl.in), perm = sorted -> original;
 *   - the Reduction tool (Reduction.cpp:143-259) for min/max of r_in and the
 *     min of dt_var, with the identities of LinkList.cpp:80-91 and
 *     cfd/variableTimeStep.xml:12;
 *   - the `copy`, `set` and `set_scalar` tools the presets use.
 * The "sums start at zero" semantics of the reference's LOCAL_MEM kernel
 * variants (Kernel.cpp:392-462) are reproduced by clearing each accumulated
 * array right before its kernel runs.
 */
#include "resources/Scripts/types/types.h"

#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>
#include <omp.h>

#include "../aqua_oracle.h"

thread_local usize aqr_gid = 0;

/* Definitions of the compiled program (CalcServer.cpp:235-264): the host
 * evaluates them and bakes them in as literals; here they are read from the
 * case parameters, with the same float values. */
struct AqrDefs
{
    float H, CONW, CONF, SUPPORT, DIMS, dr_factor, min_bound_dist;
};
static AqrDefs aqr_defs;

/* Must precede the macro definitions below (the field names collide). */
static void
aqr_set_defs(const aq_params* pr)
{
    aqr_defs = AqrDefs{ pr->H, pr->CONW, pr->CONF, pr->SUPPORT, pr->DIMS,
                        pr->dr_factor, pr->min_bound_dist };
}

#define H (aqr_defs.H)
#define CONW (aqr_defs.CONW)
#define CONF (aqr_defs.CONF)
#define SUPPORT (aqr_defs.SUPPORT)
#define DIMS (aqr_defs.DIMS)
#define __DR_FACTOR__ (aqr_defs.dr_factor)
#define __MIN_BOUND_DIST__ (aqr_defs.min_bound_dist)
#define __LAP_MONAGHAN__ 1
#define __LAP_MORRIS__ 2
#define __LAP_FORMULATION__ __LAP_MORRIS__
#define KERNEL_NAME Wendland

#include "resources/Scripts/KernelFunctions/Kernel.h"

namespace ref_midpoint {
#include "resources/Scripts/basic/time_scheme/midpoint.cl"
}
namespace ref_improved_euler {
#include "resources/Scripts/basic/time_scheme/improved_euler.cl"
}
namespace ref_domain {
#include "resources/Scripts/basic/Domain.cl"
}
namespace ref_sort {
#include "resources/Scripts/basic/Sort.cl"
}
namespace ref_eos {
#include "resources/Scripts/basic/EOS.cl"
}
#undef EXCLUDED_PARTICLE
namespace ref_binormal {
#include "resources/Scripts/basic/Binormal.cl"
}
namespace ref_shepard {
#include "resources/Scripts/cfd/Shepard.cl"
}
#undef EXCLUDED_PARTICLE
#undef _SHEPARD_
namespace ref_interactions {
#include "resources/Scripts/cfd/Interactions.cl"
}
#undef _GRADP_
#undef _LAPU_
#undef _DIVU_
namespace ref_sensors {
#include "resources/Scripts/cfd/Sensors.cl"
}
#undef _U_
#undef _RHO_
#undef _P_
namespace ref_sensors_renorm {
#include "resources/Scripts/cfd/SensorsRenormalization.cl"
}
namespace ref_deltasph {
#include "resources/Scripts/cfd/deltaSPH.cl"
}
#undef EXCLUDED_PARTICLE
#undef _GRADP_
#undef _LAPP_
namespace ref_bie_interactions {
#include "resources/Scripts/cfd/Boundary/BIe/Interactions.cl"
}
#undef _GRADW_
#undef _DIVU_
#undef _P_
namespace ref_bie_rates {
#include "resources/Scripts/cfd/Boundary/BIe/Rates.cl"
}
namespace ref_rates {
#include "resources/Scripts/cfd/Rates.cl"
}
namespace ref_elastic_bounce {
#include "resources/Scripts/cfd/Boundary/BIe/ElasticBounce.cl"
}
#undef _U_
#undef _DUDT_
namespace ref_pst {
#include "resources/Scripts/cfd/Boundary/BIe/PST.cl"
}
namespace ref_timestep {
#include "resources/Scripts/cfd/TimeStep.cl"
}
/* BI walls (cfd/BI.xml) */
namespace ref_bi_shepard {
#include "resources/Scripts/cfd/Boundary/BI/Shepard.cl"
}
#undef _SHEPARD_
namespace ref_bi_lapu {
#include "resources/Scripts/cfd/Boundary/BI/LapU.cl"
}
#undef _LAPU_
namespace ref_bi_gradp {
#include "resources/Scripts/cfd/Boundary/BI/GradP.cl"
}
namespace ref_bi_interp {
#include "resources/Scripts/cfd/Boundary/BI/Interpolation.cl"
}
#undef _P_
namespace ref_bi_interp_shepard {
#include "resources/Scripts/cfd/Boundary/BI/InterpolationShepard.cl"
}
namespace ref_bi_interactions {
#include "resources/Scripts/cfd/Boundary/BI/Interactions.cl"
}
#undef _GRADP_
#undef _DIVU_
namespace ref_linklist {
#include "aquagpusph/CalcServer/LinkList.cl.in"
}

/* ------------------------------------------------------------------------ */

namespace {

/* Run a kernel over the NDRange [0, n) */
template<typename F>
void
ndrange(usize n, int nthreads, F&& f)
{
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (long i = 0; i < (long)n; i++) {
        aqr_gid = (usize)i;
        f();
    }
}

struct Work
{
    /* usize copies of the index Variables the kernels take as usize* */
    std::vector<usize> id, id_in, icell, ihoc, id_sorted, id_unsorted;
};

usize4
ncells_of(const aq_state* st)
{
    return usize4{ st->n_cells[0], st->n_cells[1], st->n_cells[2], st->n_cells[3] };
}

/* link-list tool (LinkList::_execute) on st->r_in */
int
linklist(aq_state* st, const aq_params* pr, Work& w, int nt)
{
    const usize N = st->N;
    const vec* r_in = (const vec*)st->r_in;
    /* Reductions min/max, identities VEC_INFINITY / -VEC_INFINITY */
    vec rmin = VEC_INFINITY, rmax = VEC_NEG_INFINITY;
    for (usize i = 0; i < N; i++) {
        rmin.x = min(rmin.x, r_in[i].x);
        rmin.y = min(rmin.y, r_in[i].y);
        rmax.x = max(rmax.x, r_in[i].x);
        rmax.y = max(rmax.y, r_in[i].y);
#ifdef HAVE_3D
        rmin.z = min(rmin.z, r_in[i].z);
        rmin.w = min(rmin.w, r_in[i].w);
        rmax.z = max(rmax.z, r_in[i].z);
        rmax.w = max(rmax.w, r_in[i].w);
#endif
    }
    std::memset(st->r_min, 0, sizeof(st->r_min));
    std::memset(st->r_max, 0, sizeof(st->r_max));
    std::memcpy(st->r_min, &rmin, sizeof(vec));
    std::memcpy(st->r_max, &rmax, sizeof(vec));

    /* LinkList::nCells -- host float arithmetic, division by cell length */
    const float cell_length = pr->support * pr->h;
    if (!cell_length)
        return AQ_ERR_INVALID;
    unsigned long nx = (unsigned long)((rmax.x - rmin.x) / cell_length) + 6;
    unsigned long ny = (unsigned long)((rmax.y - rmin.y) / cell_length) + 6;
    unsigned long nz = 1;
#ifdef HAVE_3D
    nz = (unsigned long)((rmax.z - rmin.z) / cell_length) + 6;
#endif
    const unsigned long nw = nx * ny * nz;
    if (nw > st->ihoc_capacity || nw > 0xffffffffUL)
        return AQ_ERR_CAPACITY;
    st->n_cells[0] = (uint32_t)nx;
    st->n_cells[1] = (uint32_t)ny;
    st->n_cells[2] = (uint32_t)nz;
    st->n_cells[3] = (uint32_t)nw;
    const usize4 n_cells = ncells_of(st);

    /* iCell */
    w.icell.assign(N, 0);
    ndrange(N, nt, [&]() {
        ref_linklist::iCell(w.icell.data(), r_in, N, rmin, pr->support, pr->h, n_cells);
    });
    /* sort (stable), perm -> id_unsorted, inverse -> id_sorted */
    std::vector<uint32_t> keys(N), perm(N), inv(N);
    for (usize i = 0; i < N; i++)
        keys[i] = (uint32_t)w.icell[i];
    aq_sort(keys.data(), perm.data(), inv.data(), (uint32_t)N);
    w.id_unsorted.resize(N);
    w.id_sorted.resize(N);
    for (usize i = 0; i < N; i++) {
        w.icell[i] = keys[i];
        w.id_unsorted[i] = perm[i];
        w.id_sorted[i] = inv[i];
    }
    /* iHoc, linkList */
    w.ihoc.assign(nw, 0);
    ndrange(nw, nt, [&]() { ref_linklist::iHoc(w.ihoc.data(), N, n_cells); });
    if (N > 1)
        ndrange(N - 1, nt, [&]() { ref_linklist::linkList(w.icell.data(), w.ihoc.data(), N); });
    else if (N == 1)
        w.ihoc[w.icell[0]] = 0;

    for (usize i = 0; i < N; i++) {
        st->icell[i] = (uint32_t)w.icell[i];
        st->id_unsorted[i] = (uint32_t)w.id_unsorted[i];
        st->id_sorted[i] = (uint32_t)w.id_sorted[i];
    }
    for (usize c = 0; c < nw; c++)
        st->ihoc[c] = (uint32_t)w.ihoc[c];
    return AQ_OK;
}

template<typename T>
void
copy_n(const T* src, T* dst, usize n)
{
    std::memcpy(dst, src, n * sizeof(T));
}

} // namespace

extern "C" int
aq_sort(uint32_t* keys, uint32_t* perm, uint32_t* inv_perm, uint32_t n)
{
    std::vector<uint32_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0u);
    std::stable_sort(idx.begin(), idx.end(),
                     [&](uint32_t a, uint32_t b) { return keys[a] < keys[b]; });
    std::vector<uint32_t> sorted(n);
    for (uint32_t s = 0; s < n; s++) {
        sorted[s] = keys[idx[s]];
        perm[s] = idx[s];
        inv_perm[idx[s]] = s;
    }
    std::memcpy(keys, sorted.data(), n * sizeof(uint32_t));
    return AQ_OK;
}

extern "C" int
aq_linklist(aq_state* st, const aq_params* pr, int nthreads)
{
    Work w;
    return linklist(st, pr, w, nthreads > 0 ? nthreads : omp_get_max_threads());
}

extern "C" int
aq_step(aq_state* st, const aq_params* pr, int nthreads)
{
#ifdef HAVE_3D
    if (pr->dims != 3)
        return AQ_ERR_INVALID;
#else
    if (pr->dims != 2)
        return AQ_ERR_INVALID;
#endif
    const int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
    aqr_set_defs(pr);
    const usize N = st->N;
    const float dt = st->dt;
    Work w;

    vec* r = (vec*)st->r;
    vec* u = (vec*)st->u;
    vec* dudt = (vec*)st->dudt;
    vec* normal = (vec*)st->normal;
    vec* tangent = (vec*)st->tangent;
    vec* binormal = (vec*)st->binormal;
    vec* r_in = (vec*)st->r_in;
    vec* u_in = (vec*)st->u_in;
    vec* dudt_in = (vec*)st->dudt_in;
    vec* normal_in = (vec*)st->normal_in;
    vec* tangent_in = (vec*)st->tangent_in;
    vec* grad_p = (vec*)st->grad_p;
    vec* lap_u = (vec*)st->lap_u;
    vec* grad_w_bi = (vec*)st->grad_w_bi;
    vec g, domain_min, domain_max;
    std::memcpy(&g, pr->g, sizeof(vec));
    std::memcpy(&domain_min, pr->domain_min, sizeof(vec));
    std::memcpy(&domain_max, pr->domain_max, sizeof(vec));

    const bool ie = pr->scheme == 1;
    /* predictor (midpoint.cl:53-75 or improved_euler.cl:75-103) */
    if (ie) {
        ndrange(N, nt, [&]() {
            ref_improved_euler::predictor(st->imove, r, u, dudt, st->rho,
                                          st->drhodt, r_in, u_in, dudt_in,
                                          st->rho_in, st->drhodt_in, N, dt);
        });
    } else {
        ndrange(N, nt, [&]() {
            ref_midpoint::predictor(r, u, dudt, st->rho, st->drhodt, r_in,
                                    u_in, dudt_in, st->rho_in, st->drhodt_in,
                                    N);
        });
    }
    /* Domain (Domain.cl:48-90) */
    ndrange(N, nt, [&]() {
        ref_domain::entry(st->imove, r_in, u_in, dudt_in, st->m, N, domain_min,
                          domain_max);
    });
    /* link-list on r_in */
    int err = linklist(st, pr, w, nt);
    if (err)
        return err;
    const usize4 n_cells = ncells_of(st);
    const usize* icell = w.icell.data();
    const bool bi = pr->boundary == 1;
    /* 32-bit copies for the kernel that declares uint link-list arguments
     * (BI/Interactions.cl) */
    std::vector<uint> icell32(w.icell.begin(), w.icell.end());
    std::vector<uint> ihoc32(w.ihoc.begin(), w.ihoc.end());
    const uint4 n_cells32{ (uint)n_cells.x, (uint)n_cells.y, (uint)n_cells.z,
                           (uint)n_cells.w };
    const usize* ihoc = w.ihoc.data();
    /* Backup id, iset, imove, normal, tangent, m (basic.xml:141-146) */
    w.id.resize(N);
    w.id_in.resize(N);
    for (usize i = 0; i < N; i++)
        w.id_in[i] = st->id[i];
    copy_n(st->iset, st->iset_in, N);
    copy_n(st->imove, st->imove_in, N);
    copy_n(normal, normal_in, N);
    copy_n(tangent, tangent_in, N);
    copy_n(st->m, st->m_in, N);
    copy_n(st->id, st->id_in, N);
    /* sort stage1 / stage2 (Sort.cl:57-124) */
    ndrange(N, nt, [&]() {
        ref_sort::stage1(w.id_in.data(), w.id.data(), st->iset_in, st->iset,
                         st->imove_in, st->imove, r_in, r, normal_in, normal,
                         tangent_in, tangent, w.id_sorted.data(), N);
    });
    for (usize i = 0; i < N; i++)
        st->id[i] = (uint32_t)w.id[i];
    ndrange(N, nt, [&]() {
        ref_sort::stage2(st->rho_in, st->rho, st->m_in, st->m, u_in, u, dudt,
                         dudt_in, st->drhodt, st->drhodt_in,
                         w.id_sorted.data(), N);
    });
    /* EOS, Binormal */
    ndrange(N, nt, [&]() {
        ref_eos::entry(st->iset, st->imove, st->rho, st->p, pr->refd, N, pr->cs,
                       pr->p0);
    });
    ndrange(N, nt, [&]() { ref_binormal::entry(normal, tangent, binormal, N); });
    /* cfd / deltaSPH reinit sets (cfd.xml:59-62, deltaSPH.xml:31) */
    std::fill(st->lap_p, st->lap_p + N, 0.f);
    std::fill(lap_u, lap_u + N, VEC_ZERO);
    std::fill(st->div_u, st->div_u + N, 0.f);
    std::fill(grad_p, grad_p + N, VEC_ZERO);
    std::fill(st->shepard, st->shepard + N, 0.f);
    /* midpoint init (midpoint.xml); the improved Euler scheme has no loop
     * and none of these tools: the sweeps run once on the sorted predictor
     * output */
    if (!ie) {
        copy_n(st->drhodt_in, st->drhodt, N);
        copy_n(dudt_in, dudt, N);
        copy_n(r, r_in, N);
        copy_n(u, u_in, N);
        copy_n(st->rho, st->rho_in, N);
    }
    const uint32_t passes = ie ? 1u : pr->iter_midpoint_max;
    for (uint32_t iter_midpoint = 0; iter_midpoint < passes; iter_midpoint++) {
        if (!ie) {
            copy_n(st->drhodt, st->drhodt_in, N);
            copy_n(dudt, dudt_in, N);
            ndrange(N, nt, [&]() {
                ref_midpoint::midpoint(st->imove, u_in, u, dudt, st->rho_in,
                                       st->rho, st->drhodt, N, dt);
            });
            ndrange(N, nt, [&]() {
                ref_eos::entry(st->iset, st->imove, st->rho, st->p, pr->refd,
                               N, pr->cs, pr->p0);
            });
        }
        /* neighbour sweeps; LOCAL_MEM semantics: sums start at zero */
        std::fill(st->shepard, st->shepard + N, 0.f);
        if (bi) {
            /* cfd Shepard replaced by the analytic BI factor (BI.xml:33) */
            ndrange(N, nt, [&]() {
                ref_bi_shepard::compute(st->imove, r, normal, tangent, binormal,
                                        st->m, st->shepard, N, icell, ihoc,
                                        n_cells);
            });
        } else {
            ndrange(N, nt, [&]() {
                ref_shepard::entry(st->imove, r, st->rho, st->m, st->shepard, N,
                                   icell, ihoc, n_cells);
            });
        }
        std::fill(grad_p, grad_p + N, VEC_ZERO);
        std::fill(lap_u, lap_u + N, VEC_ZERO);
        std::fill(st->div_u, st->div_u + N, 0.f);
        ndrange(N, nt, [&]() {
            ref_interactions::entry(st->imove, r, u, st->rho, st->m, st->p,
                                    grad_p, lap_u, st->div_u, N, icell, ihoc,
                                    n_cells);
        });
        ndrange(N, nt, [&]() {
            ref_sensors::entry(st->iset, st->imove, r, st->m, u, st->rho,
                               st->p, N, g, icell, ihoc, n_cells);
        });
        ndrange(N, nt, [&]() {
            ref_sensors_renorm::entry(st->imove, st->shepard, u, st->rho,
                                      st->p, N, dt, g);
        });
        std::fill(st->lap_p, st->lap_p + N, 0.f);
        ndrange(N, nt, [&]() {
            ref_deltasph::lapp(st->imove, r, st->rho, st->m, st->p, st->lap_p,
                               N, icell, ihoc, n_cells);
        });
        if (bi) {
            /* BI.xml:24-32, in insertion order before "Interactions" */
            ndrange(N, nt, [&]() {
                ref_bi_lapu::freeslip(st->imove, r, u, st->rho, st->m, lap_u,
                                      N, icell, ihoc, n_cells);
            });
            ndrange(N, nt, [&]() {
                ref_bi_gradp::freeslip(st->iset, st->imove, st->shepard,
                                       st->rho, lap_u, dudt, grad_p,
                                       pr->visc_dyn, pr->refd, N, g);
            });
            ndrange(N, nt, [&]() {
                ref_bi_interp::entry(st->iset, st->imove, r, st->m, st->rho,
                                     grad_p, st->p, pr->refd, N, icell, ihoc,
                                     n_cells);
            });
            ndrange(N, nt, [&]() {
                ref_bi_interp_shepard::entry(st->iset, st->imove, st->shepard,
                                             st->rho, st->p, pr->refd, N,
                                             pr->cs, pr->p0);
            });
            ndrange(N, nt, [&]() {
                ref_bi_interactions::entry(st->iset, st->imove, r, normal, u,
                                           st->rho, st->m, st->p, pr->refd,
                                           grad_p, st->div_u, icell32.data(),
                                           ihoc32.data(), N, n_cells32, g);
            });
            ndrange(N, nt, [&]() {
                ref_bi_shepard::apply(st->imove, st->shepard, grad_p, lap_u,
                                      st->div_u, N, pr->cs);
            });
        } else {
            std::fill(grad_w_bi, grad_w_bi + N, VEC_ZERO);
            std::fill(st->div_u_bi, st->div_u_bi + N, 0.f);
            ndrange(N, nt, [&]() {
                ref_bie_interactions::entry(st->imove, r, normal, u, st->m,
                                            grad_w_bi, st->div_u_bi, N, icell,
                                            ihoc, n_cells);
            });
            ndrange(N, nt, [&]() {
                ref_bie_rates::entry(st->imove, st->rho, st->p, u, grad_w_bi,
                                     st->div_u_bi, grad_p, st->div_u, N);
            });
        }
        ndrange(N, nt, [&]() {
            ref_rates::entry(st->iset, st->imove, st->rho, grad_p, lap_u,
                             st->div_u, dudt, st->drhodt, pr->visc_dyn, N, g);
        });
        ndrange(N, nt, [&]() {
            ref_deltasph::deltaSPH(st->iset, st->imove, st->rho, st->lap_p,
                                   st->drhodt, pr->refd, pr->delta, N, dt);
        });
        if (!bi) {
            ndrange(N, nt, [&]() {
                ref_elastic_bounce::entry(st->imove, r_in, normal, st->m, u_in,
                                          dudt, N, dt, icell, ihoc, n_cells);
            });
        }
        if (!ie) {
            ndrange(N, nt, [&]() {
                ref_midpoint::relax(st->imove, dudt_in, dudt, st->drhodt_in,
                                    st->drhodt, N, pr->relax_midpoint);
            });
        }
    }
    /* corrector (midpoint.cl:206-227 or improved_euler.cl:125-147), PST */
    if (ie) {
        ndrange(N, nt, [&]() {
            ref_improved_euler::corrector(st->imove, st->iset, r, u, dudt,
                                          st->rho, st->drhodt, dudt_in,
                                          st->drhodt_in, N, dt);
        });
    } else {
        ndrange(N, nt, [&]() {
            ref_midpoint::corrector(st->imove, r_in, r, u_in, u, dudt,
                                    st->rho_in, st->rho, st->drhodt, N, dt);
        });
    }
    if (!bi) {
        ndrange(N, nt, [&]() {
            ref_pst::entry(st->imove, r, normal, st->m, st->rho, N, icell,
                           ihoc, n_cells);
        });
    }
    /* fixed time step, variable time step, minimum time step (reduction) */
    const float dt_fixed = pr->dt_fixed;
    ndrange(N, nt, [&]() {
        ref_timestep::entry(st->imove, u, st->dt_var, N, dt_fixed, pr->dt_min,
                            pr->courant, pr->dt_Ma, pr->h);
    });
    float dt_new = INFINITY;
    for (usize i = 0; i < N; i++)
        dt_new = min(dt_new, st->dt_var[i]);
    if (!(dt_new > 0.f))
        return AQ_ERR_DT;
    /* t = t + dt, iter += 1 (set_scalar, evaluated in double) */
    st->dt = dt_new;
    st->t = (float)((double)st->t + (double)dt_new);
    st->iter += 1;
    return AQ_OK;
}
