/*
 * ORACLE — test infrastructure, not product code.
 *
 * C-ABI of the CPU restatement of InterfaceAdvection.jl's per-step hot path
 * (oracle.cpp).  Only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / `--impl reference` arm load this library, and only as the
 * checker or as the timed CPU baseline.  The product library
 * (libintfadv_gb300.so) never links or calls it.
 *
 * Memory layout is the reference's Julia layout: column-major (x fastest),
 * one ghost layer on every side (Ng = N + 2), vector fields SoA with the
 * component index last (component d starts at d * Ng_total).  Indices are
 * 0-based: Julia index k is k-1 here.
 */
#ifndef INTFADV_ORACLE_H
#define INTFADV_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int32_t D;      /* 2 or 3 */
    int32_t per;    /* bit j set <=> dimension j (0-based) is periodic */
    int64_t n[3];   /* ghost-inclusive sizes, n[2] = 1 when D == 2 */
} orc_grid;

/* reportFillError (src/advection.jl:145-189) outcome of the last sweep that flagged. */
typedef struct {
    int32_t nan;        /* error("NaN!") */
    int32_t over;       /* max f - 1 > tol (printed by the reference, not fatal) */
    int32_t under;      /* min f < -tol   (printed, not fatal) */
    int32_t diverge;    /* |div u0| + |div u| > 10 at the offending cell (fatal) */
    int32_t dir;        /* 0-based sweep direction of the last flag */
    int32_t pad;
    double  maxf, minf;
    int64_t maxid, minid;
} orc_fill_status;

/* Normal schemes (src/normalEstimation.jl), same numbering as the product ABI. */
enum { ORC_WH = 0, ORC_WY = 1, ORC_MYC = 2, ORC_Y = 3, ORC_COLUMN = 4,
       ORC_PCD = 5, ORC_SLIC = 6, ORC_CD = 7, ORC_XYLIC = 8 };
/* Limiters (src/flow.jl:5-15). */
enum { ORC_KOREN = 0, ORC_UPWIND = 1, ORC_MINMOD = 2, ORC_VANALBADA1 = 3,
       ORC_SWEBY = 4, ORC_SUPERBEE = 5, ORC_TVDCEN = 6, ORC_TVDDOWN = 7 };

/* ---- PLIC (src/PLIC.jl) -------------------------------------------------- */
double orc_get_intercept2(double n1, double n2, double g);
double orc_get_intercept3(double n1, double n2, double n3, double g);
double orc_get_volume_fraction2(double n1, double n2, double b);
double orc_get_volume_fraction3(double n1, double n2, double n3, double b);
float  orc_get_intercept2f(float n1, float n2, float g);
float  orc_get_intercept3f(float n1, float n2, float n3, float g);
float  orc_get_volume_fraction2f(float n1, float n2, float b);
float  orc_get_volume_fraction3f(float n1, float n2, float n3, float b);
double orc_proot(double c0, double c1, double c2, double c3);

/* ---- util / VOFutil ------------------------------------------------------ */
int    orc_normal(const orc_grid* g, int scheme, const double* f, double* nhat, int64_t I);
void   orc_reconstruct(const orc_grid* g, int scheme, const double* f, double* alpha, double* nhat);
void   orc_bcvof(const orc_grid* g, double* f, double* alpha, double* nhat);
void   orc_bcf(const orc_grid* g, double* f);
void   orc_bcf_d(const orc_grid* g, int d, double* f);
void   orc_bcv(const orc_grid* g, double* v);
void   orc_bc_vel(const orc_grid* g, double* a, const double* A);   /* WaterLily BC! (constant A) */
void   orc_perbc(const orc_grid* g, double* x);                     /* WaterLily perBC! */
void   orc_clean_wisp(const orc_grid* g, double* f, double tol);
void   orc_f2face(const orc_grid* g, double* fface, const double* f);
double orc_get3cellheight(const orc_grid* g, const double* f, int64_t I, int s);
double orc_getmu(const orc_grid* g, int i, int j, int64_t I, const double* fface,
                 double lmu, double mu, double lrho);
/* applyVOF! (src/VOFutil.jl:9-37) from SDF samples: sdf[0] = centre, sdf[1+2d] = +0.01 e_d,
 * sdf[2+2d] = -0.01 e_d; each a scalar field. */
void   orc_apply_vof(const orc_grid* g, double* f, double* alpha, double* nhat,
                     const double* const* sdf);

/* ---- VOF advection (src/advection.jl) ------------------------------------ */
void   orc_vof_flux(const orc_grid* g, double* fF, const double* f, const double* alpha,
                    const double* nhat, const double* u, const double* u0, double dt,
                    int d, double* rhouf, double lrho);
void   orc_advect_vof(const orc_grid* g, int scheme, double* f, double* fF, double* alpha,
                      double* nhat, const double* u, const double* u0, double dt,
                      int8_t* cbar, double* rhouf, double lrho, const int* dirO,
                      orc_fill_status* st);

/* ---- surface tension (src/surfaceTension.jl) ----------------------------- */
double orc_popinet_height(const orc_grid* g, const double* f, int64_t I, int i_signed);
double orc_curvature(const orc_grid* g, const double* f, int64_t I, int i_signed);
/* surfTen!(forcing, f, α, n̂, fbuffer, η) (src/surfaceTension.jl:8-20): fbuffer is the caller's
 * buffer, reused for every d exactly as the reference does (its high ghost along a wall d keeps the
 * previous content); n̂ receives the WY normals. */
void   orc_surften(const orc_grid* g, double* forcing, const double* f, double* nhat, double* fbuffer,
                   double eta);

/* ---- full two-phase step (src/flow.jl) ----------------------------------- */
typedef struct {
    /* Flow (WaterLily) */
    double *u, *u0, *force, *sigma, *p, *mu0;
    /* Poisson work arrays (scalars) */
    double *pr, *peps, *pz, *pD, *piD;
    /* cVOF */
    double *f, *f0, *alpha, *nhat, *fF, *rhou, *rhouf, *drho;
    int8_t *cbar;
    double lrho, lmu;
    double mu;          /* 0 => viscosity off (cVOF stores `nothing`) */
    double eta;         /* 0 => surface tension off */
    double nu;          /* WaterLily ν used by MPCFL */
    double g[3];        /* constant gravity */
    int32_t has_g;
    int32_t scheme;     /* normal scheme */
    int32_t limiter;
    int32_t pad;
    double uBC[3];      /* constant boundary velocity */
    /* Poisson controls */
    double ptol;        /* L-infinity residual tolerance of the dt-scaled system */
    int32_t pitmx;
    int32_t piters;     /* out: PCG iterations of the last solve */
    double presid;      /* out: final L-infinity residual */
    int32_t psolver;    /* ORC_POISSON_JACOBI (psolver!, flow.jl:300-326) or ORC_POISSON_MG
                           (multigrid-preconditioned CG in the role of MultiLevelPoisson, :343-347) */
    int32_t pad2;
} orc_state;
enum { ORC_POISSON_JACOBI = 0, ORC_POISSON_MG = 1 };

void   orc_mom_step(const orc_grid* g, orc_state* s, double dt, double t_now,
                    int64_t n_dt, orc_fill_status* st);
double orc_mpcfl(const orc_grid* g, orc_state* s, double dt_last);
void   orc_poisson(const orc_grid* g, orc_state* s);

/* ---- helpers for known-answer tests ---- */
int    orc_argabsmax(int D, const double* n);
int    orc_get_xdir(int i);
void   orc_get_xydir(int i, int* ix, int* iy);
double orc_getrho_cell(double f, double lrho);
double orc_getrho_face(const orc_grid* g, int d, int64_t I, const double* f, double lrho);
void   orc_vof_flux_face(const orc_grid* g, double* fF, const double* f, const double* alpha,
                         const double* nhat, double dl, int d, int64_t IFace, double* rhouf, double lrho);

#ifdef __cplusplus
}
#endif
#endif
