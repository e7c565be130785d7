/*
 * CPU oracle for the snapy MeshBlock hydro stage -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C FP64 restatement of the reference's algorithm, used by tests/,
 * __graft_entry__.smoke() and the cpu_baseline leg of bench.py as the checker.
 * Nothing in the product (snapy_gb300/) may call it.
 *
 * Layout: every cell field is (nvar, nc3, nc2, nc1), x1 contiguous, exactly as
 * the reference's hydro_u / hydro_w (src/snap.h:34-46 row order IDN, IVX, IVY,
 * IVZ, IPR).
 */
#ifndef SG_ORACLE_H
#define SG_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { OG_IDN = 0, OG_IVX = 1, OG_IVY = 2, OG_IVZ = 3, OG_IPR = 4 };
enum { OG_HLLC = 0, OG_LMARS = 1 };
enum {
  OG_BC_NONE = 0,        /* no boundary function (custom no-op) */
  OG_BC_REFLECTING = 1,
  OG_BC_PERIODIC = 2,
  OG_BC_EXTRAPOLATION = 3
};

typedef struct og_block {
  int nvar;            /* 5 */
  int nc1, nc2, nc3;   /* padded sizes (nx + 2 ng on an active axis, else 1) */
  int ng;              /* ghost width, 3 */
  double dx1, dx2, dx3;
  double x1min, x2min, x3min; /* lower bound of the interior */
  double gammad;
  int riemann;         /* OG_HLLC / OG_LMARS */
  int shock;           /* 1: every row weno5; 0: IDN weno5, IVX..IPR cp5 */
  int weno_scale;      /* InterpOptions::scale */
  int bc[6];           /* x1-inner, x1-outer, x2-inner, x2-outer, x3-in, x3-out */
  /* RK3 weights (w0, w1, w2) per stage: u <- w0 u0 + w1 u + w2 du */
  double wght[3][3];
  int nthreads;        /* OpenMP threads, 0 = default */
  /* the Straka-class physics (0 = off) */
  double grav1;        /* forcing/const-gravity/grav1 (x1 acceleration) */
  double nu_iso;       /* forcing/diffusion/nu_iso (kinematic viscosity) */
  int flux_cov;        /* dynamics/flux-covariance */
  int wb_wall_clamp;   /* dynamics/wb-wall-clamp */
  int implicit_scheme; /* integration/implicit-scheme: 0 off, 9 full 5x5,
                          1 partial 3x3 */
  double cfl;          /* integration/cfl (the implicit x1 time-step rule) */
  /* geometry of the padded block: x1f[nc1 + 1], x1v[nc1] (the reference's
   * linspace faces), x2v[nc2] */
  const double* x1f;
  const double* x1v;
  const double* x2v;
  /* the FluxRegister's FP64 step fields S_d (5, nc3, nc2, nc1), face f along
   * d below cell f, updated by og_stage on the faces of the interior cells
   * (NULL: not requested), and, when set, the stage's face totals T_d on the
   * same faces (FluxRegister::total after HydroImpl::forward) */
  double* step[3];
  double* total[3];
  /* scalar/nvar passive scalars (src/scalar/scalar.cpp:90-211): their
   * densities (nscalar, nc3, nc2, nc1), advanced in place by og_stage, and
   * the stage-0 backup; nscalar 0 or scalar NULL: none */
  int nscalar;
  double* scalar;
  double* scalar0;
  /* og_stage's scratch for the implicit solve's face transfers (the
   * scalars' share of them): the clamped dry transfer q of each x1 face,
   * face f below cell f; set by og_stage itself */
  double* vic_q;
  /* the RegisterMonitor count this path can raise in the stage
   * (src/riemann/riemann.cpp:330-339): monitor[0] += the interior faces
   * whose HLLC contact pressure was clamped to zero (riemann.pstar_clamp);
   * NULL: not counted */
  long long* monitor;
} og_block;

/* ---- unit functions (pinned against the reference headers) ---- */
/* one WENO5 face from 5 consecutive cells; side 0 = the cm table (the state on
 * the right of the lower face of the centre cell), 1 = the cp table */
double og_weno5_face(const double* s5, int side, int scale);
double og_cp5_face(const double* s5, int side);
/* HLLC / LMARS flux at one face from two primitive states (nvar 5) */
void og_hllc_face(const double* wl, const double* wr, double gammad, int dim,
                  double* flx, double* face_pressure);
void og_lmars_face(const double* wl, const double* wr, double gammad, int dim,
                   double* flx, double* face_pressure);
void og_cons2prim_cell(const double* u, double* w, double gammad, int stride);

/* the portable exp of the reference anchor (same operations as the GPU) */
double og_exp(double x);

/* ---- block operations ---- */
void og_default_block(og_block* b);
void og_cons2prim(const og_block* b, const double* u, double* w);
void og_prim2cons(const og_block* b, const double* w, double* u);
/* boundary functions, faces in order 0..5; primitive selects kPrimitive */
void og_apply_bc(const og_block* b, double* q, int primitive);
/* the kScalar boundary functions on nscalar rows of tracer densities */
void og_scalar_bc(const og_block* b, double* s);
/* face fluxes of direction d (1 = x1, 2 = x2, 3 = x3) at every face */
void og_flux(const og_block* b, const double* w, int d, double* flux);
/* one RK stage: u is advanced in place; u0 holds the stage-0 backup */
void og_stage(const og_block* b, double* u, double* u0, double dt, int stage);
/* the hydro tendency of one stage (HydroImpl::forward): du on every cell
 * (zero outside the interior), from the primitives w */
void og_tendency(const og_block* b, const double* w, double dt, double* du);
/* the vertical implicit correction (scheme 9, or 1: the partial matrix) of
 * every interior column:
 * du (the explicit tendency, gravity work included) is replaced by the
 * corrected one; dtc = wght2 dt.  Returns the number of failed columns
 * (their du is left as it came in) */
int og_implicit(const og_block* b, const double* w, double dtc, double* du);
/* the same, posting the solve's x1 face transfers into the register total
 * t1 (5, nc3, nc2, nc1) with the step's dt (null t1: none) */
int og_implicit_reg(const og_block* b, const double* w, double dtc, double* du,
                    double* t1, double dt);
/* the partial matrix's redistribution of one column alone (constituent
 * column, tangential momenta, per-cell map): n layers, w and du 5 x n,
 * vol[n], delta n x 3 (total mass, m1, E) */
void og_vic_redistribute_partial(int n, const double* w, double* du,
                                 const double* vol, const double* delta);
/* the well-balanced x1 reference of one column (w strided by `plane`):
 * psf_lo, psf_hi, pref, dsf, dref [nc1] and dsf_lr [2][nc1] */
void og_ref_column(const og_block* b, const double* w, size_t plane,
                   double* psf_lo, double* psf_hi, double* pref, double* dsf,
                   double* dref, double* dsf_lr);
/* the hydro time step (before cfl), reference HydroImpl::max_time_step */
double og_max_dt(const og_block* b, const double* w);
/* initialize: boundaries on w, W->U, boundaries on u */
void og_initialize(const og_block* b, double* w, double* u);

/* batched face helpers of the cubed-sphere oracle (oracle/cubed_sphere.py) */
void og_recon_batch(const double* st, long n, int weno, int side, int scale,
                    double* out);
void og_shallow_roe_batch(const double* wl, const double* wr, long n, int dim,
                          double* flx);
void og_hllc_sw_batch(const double* wl, const double* wr, long n, int dim,
                      double* flx);

#ifdef __cplusplus
}
#endif
#endif
