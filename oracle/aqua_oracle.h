/*
 * Host-side data contract shared by the two CPU oracles of this repository.
 * TEST INFRASTRUCTURE ONLY (the product never includes or links it):
 *
 *   liboracle.so          -- oracle/aqua_oracle.cpp: an independent C++
 *                            restatement of the reference's per-step WCSPH
 *                            pipeline (compiled on every machine, including
 *                            the GPU host, by __graft_entry__.build()).
 *   _ref/libaqua_ref2d.so  -- oracle/refshim/ref_kernels.cpp: the reference's
 *   _ref/libaqua_ref3d.so     own OpenCL kernel sources compiled as C++ on the
 *                            host (only where the reference tree is present).
 *
 * Both export the same functions over the same structs, so a test can run the
 * same state through either and compare.  Arrays follow the reference's
 * Variables layout: `vec` arrays hold VS floats per particle (VS = 4 in 3-D,
 * 2 in 2-D, i.e. float4 / float2); index arrays hold unsigned 32-bit values
 * (the reference's 32-bit-device `usize`, CalcServer.cpp:260-264).
 */
#ifndef AQUA_ORACLE_H
#define AQUA_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Constants of one case: the Variables and Definitions the canonical preset
 * stack (basic + midpoint + domain + cfd + deltaSPH + BIe + variableTimeStep)
 * binds into the kernels. */
typedef struct
{
    int32_t dims;      /* 2 or 3 */
    uint32_t n_sets;   /* length of refd / visc_dyn / delta */
    float h;           /* Variable h */
    float support;     /* Variable support */
    float H;           /* Definition H, as compiled ("%#G" of h) */
    float CONW;        /* Definition CONW = 1/h^dims, as compiled */
    float CONF;        /* Definition CONF = 1/h^(dims+2), as compiled */
    float SUPPORT;     /* Definition SUPPORT (2.f) */
    float DIMS;        /* Definition DIMS, as compiled */
    float cs;          /* Variable cs */
    float p0;          /* Variable p0 */
    float g[4];        /* Variable g */
    float courant;     /* Variable courant */
    float dt_Ma;       /* Variable dt_Ma */
    float dt_min;      /* Variable dt_min */
    float dt_fixed;    /* "fixed time step" set_scalar: courant*h/cs */
    float domain_min[4];
    float domain_max[4];
    float dr_factor;       /* Definition __DR_FACTOR__ */
    float min_bound_dist;  /* Definition __MIN_BOUND_DIST__ */
    float relax_midpoint;  /* Variable relax_midpoint */
    uint32_t iter_midpoint_max; /* Variable iter_midpoint_max */
    const float* refd;
    const float* visc_dyn;
    const float* delta;
    /* wall formulation: 0 = BIe (cfd/BIe.xml, the canonical stack), 1 = BI
     * (cfd/BI.xml: analytic Shepard, free-slip boundary integrals) */
    int32_t boundary;
    /* time scheme: 0 = midpoint (basic/time_scheme/midpoint.xml), 1 =
     * improved Euler (basic/time_scheme/improved_euler.xml); only the
     * reference-kernel harness runs 1 */
    int32_t scheme;
    /* prescribed roll of the boundary elements and probes (non-fluid
     * particles of set roll_iset) about z through roll_center:
     * psi(t) = roll_amplitude * sin(roll_angular_freq * t), applied after the
     * time step (cfd/motion.xml:59-71); the reference-kernel harness ignores
     * these fields */
    int32_t roll_enabled;
    uint32_t roll_iset;
    float roll_amplitude;
    float roll_angular_freq;
    float roll_center[4];
} aq_params;

/* Particle Variables (host pointers). */
typedef struct
{
    uint32_t N;
    uint32_t ihoc_capacity; /* allocated length of ihoc */
    /* state */
    uint32_t* id;
    uint32_t* iset;
    int32_t* imove;
    float* r;
    float* normal;
    float* tangent;
    float* binormal;
    float* u;
    float* dudt;
    float* rho;
    float* drhodt;
    float* m;
    float* p;
    /* backups written by a step */
    uint32_t* id_in;
    uint32_t* iset_in;
    int32_t* imove_in;
    float* r_in;
    float* normal_in;
    float* tangent_in;
    float* u_in;
    float* dudt_in;
    float* rho_in;
    float* drhodt_in;
    float* m_in;
    /* intermediate fields of a step */
    float* grad_p;
    float* lap_u;
    float* div_u;
    float* shepard;
    float* lap_p;
    float* grad_w_bi;
    float* div_u_bi;
    float* dt_var;
    /* link-list */
    uint32_t* icell;
    uint32_t* id_sorted;
    uint32_t* id_unsorted;
    uint32_t* ihoc;
    /* scalars */
    float r_min[4];
    float r_max[4];
    uint32_t n_cells[4];
    float t;
    float dt;
    uint32_t iter;
} aq_state;

/* Status codes (shared with the CUDA library) */
#define AQ_OK 0
#define AQ_ERR_INVALID (-1)
#define AQ_ERR_CAPACITY (-2)
#define AQ_ERR_DT (-3)

/* link-list tool on st->r_in (LinkList.cpp:326-494): r_min/r_max, n_cells,
 * icell (sorted), id_sorted, id_unsorted, ihoc. */
int aq_linklist(aq_state* st, const aq_params* pr, int nthreads);
/* stable sort of 32-bit keys (RadixSort tool, RadixSort.cpp:130-304):
 * keys sorted in place, perm[s] = original index, inv_perm[orig] = s. */
int aq_sort(uint32_t* keys, uint32_t* perm, uint32_t* inv_perm, uint32_t n);
/* one full canonical step (predictor ... t += dt) */
int aq_step(aq_state* st, const aq_params* pr, int nthreads);

#ifdef __cplusplus
}
#endif

#endif
