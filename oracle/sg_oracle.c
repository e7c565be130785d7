/*
 * CPU oracle for the snapy MeshBlock hydro stage -- TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C and FP64, the reference algorithm of one RK
 * stage of snapy's MeshBlock (a CPU restatement, not a copy).  It is the
 * checker for the CUDA product: only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py load it.  Every step keeps
 * the reference's order of floating-point operations so that the FP64 CUDA
 * path can be compared at relative L2 1e-12 (it is compiled with
 * -ffp-contract=off: the reference's torch CPU ops are not contracted).
 *
 * Reference files restated (paths inside the snapy project):
 *   src/recon/recon_point.h:44-153      weno5_point, poly_point
 *   src/recon/reconstruct.cpp:49-93     coefficient tables cm / cp
 *   src/recon/reconstruct.cpp:217-229   _apply_inplace (face indexing, ghost
 *                                       faces copy the end faces)
 *   src/recon/reconstruct.cpp:252-333   ReconstructImpl::forward (row groups)
 *   src/riemann/riemann_kernels.h:56-194  hllc_impl
 *   src/riemann/riemann_kernels.h:197-255 lmars_impl
 *   src/riemann/riemann.cpp:219-262     the EOS face pass (e, gamma, c)
 *   src/eos/ideal_gas_impl.h:16-35      ideal_gas_cons2prim
 *   src/eos/ideal_gas.cpp:53-70         _prim2cons
 *   src/coord/coordinate.cpp:618-662    divergence (area-weighted)
 *   src/coord/coordinate.cpp:488-515    Cartesian face areas and volumes
 *   src/hydro/hydro_forward.cpp:983-985 du = -dt div on the interior
 *   src/layout/seam_register.cpp:184-239, src/hydro/flux_register.cpp:700-740
 *                                       wall faces: rows IDN, IPR zeroed
 *   src/bc/bc_func.cpp:10-70            reflecting / periodic / extrapolation
 *   src/mesh/meshblock_exchange.cpp:214-286 face order of apply_boundaries
 *   src/mesh/meshblock.cpp:306-420      initialize: BC(w), W->U, BC(u)
 *   src/hydro/hydro.cpp:316-398         max_time_step (no implicit scheme)
 *   pyharp Integrator (third party, not in the reference tree): SSP-RK3
 *     u <- w0 u0 + w1 u + w2 du, w2 pinned at (1, 1/4, 2/3) by
 *     tests/test_forcing.cpp:1316-1322; w0, w1 restated as Shu-Osher.
 */
#include "sg_oracle.h"

#include <float.h>
#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define SQR(x) ((x) * (x))
#define IDX(b, v, k, j, i) \
  ((((size_t)(v) * (b)->nc3 + (k)) * (b)->nc2 + (j)) * (b)->nc1 + (i))

/* ------------------------------------------------------------------ */
/* coefficient tables, reconstruct.cpp:49-93 (cm), cp = rows flipped    */
/* ------------------------------------------------------------------ */
static const double kWeno5Rows[9][5] = {
    {-1. / 6., 5. / 6., 1. / 3., 0., 0.}, {0., 1. / 3., 5. / 6., -1. / 6., 0.},
    {0., 0., 11. / 6., -7. / 6., 1. / 3.}, {1., -2., 1., 0., 0.},
    {1., -4., 3., 0., 0.},                  {0., 1., -2., 1., 0.},
    {0., -1., 0., 1., 0.},                  {0., 0., 1., -2., 1.},
    {0., 0., 3., -4., 1.}};
static const double kWeno5D[3] = {.3, .6, .1};
static const double kCp5Cm[5] = {-1. / 20., 9. / 20., 47. / 60., -13. / 60.,
                                 1. / 30.};

static double g_weno5_cm[48], g_weno5_cp[48], g_cp5_cm[5], g_cp5_cp[5];
static int g_tables_ready = 0;

static void build_tables(void) {
  if (g_tables_ready) return;
  for (int r = 0; r < 9; ++r)
    for (int k = 0; k < 5; ++k) {
      g_weno5_cm[r * 5 + k] = kWeno5Rows[r][k];
      g_weno5_cp[r * 5 + k] = kWeno5Rows[r][4 - k];
    }
  for (int k = 0; k < 3; ++k) g_weno5_cm[45 + k] = g_weno5_cp[45 + k] = kWeno5D[k];
  for (int k = 0; k < 5; ++k) {
    g_cp5_cm[k] = kCp5Cm[k];
    g_cp5_cp[k] = kCp5Cm[4 - k];
  }
  g_tables_ready = 1;
}

/* recon_point.h:44-51 */
static double vvdot5(const double* v1, const double* v2) {
  double out = 0.;
  for (int i = 0; i < 5; ++i) out += v1[i] * v2[i];
  return out;
}

/* recon_point.h:114-147, weno5_point on a contiguous 5-cell stencil */
static double weno5_point(const double* src, int stride, const double* c,
                          int scale) {
  double phi[5];
  double vscale = 1.0;
  if (scale) {
    double sum = fabs(src[0]);
    for (int k = 1; k < 5; ++k) sum += fabs(src[k * stride]);
    vscale = sum / 5.;
  }
  if (vscale != 0.)
    for (int k = 0; k < 5; ++k) phi[k] = src[k * stride] / vscale;
  if (vscale == 0.) return 0.;
  const double *c1 = c, *c2 = c + 5, *c3 = c + 10, *c4 = c + 15, *c5 = c + 20,
               *c6 = c + 25, *c7 = c + 30, *c8 = c + 35, *c9 = c + 40;
  double p0 = vvdot5(phi, c1), p1 = vvdot5(phi, c2), p2 = vvdot5(phi, c3);
  double t;
  double beta0, beta1, beta2;
  t = vvdot5(phi, c4);
  beta0 = (13. / 12.) * SQR(t);
  t = vvdot5(phi, c5);
  beta0 = beta0 + .25 * SQR(t);
  t = vvdot5(phi, c6);
  beta1 = (13. / 12.) * SQR(t);
  t = vvdot5(phi, c7);
  beta1 = beta1 + .25 * SQR(t);
  t = vvdot5(phi, c8);
  beta2 = (13. / 12.) * SQR(t);
  t = vvdot5(phi, c9);
  beta2 = beta2 + .25 * SQR(t);
  const double* d = c9 + 5;
  const double eps = 1e-6;
  double alpha0 = d[0] / SQR(beta0 + eps);
  double alpha1 = d[1] / SQR(beta1 + eps);
  double alpha2 = d[2] / SQR(beta2 + eps);
  return vscale * (alpha0 * p0 + alpha1 * p1 + alpha2 * p2) /
         (alpha0 + alpha1 + alpha2);
}

/* recon_point.h:53-61 */
static double poly5_point(const double* src, int stride, const double* c) {
  double out = 0.;
  for (int k = 0; k < 5; ++k) out += c[k] * src[k * stride];
  return out;
}

double og_weno5_face(const double* s5, int side, int scale) {
  build_tables();
  return weno5_point(s5, 1, side ? g_weno5_cp : g_weno5_cm, scale);
}

double og_cp5_face(const double* s5, int side) {
  build_tables();
  return poly5_point(s5, 1, side ? g_cp5_cp : g_cp5_cm);
}

/* ------------------------------------------------------------------ */
/* Riemann face functions                                             */
/* ------------------------------------------------------------------ */
typedef struct {
  int x, y, z;
} axes_t;

/* riemann_kernels.h:34-38, face_axes: dim is the tensor axis (3 = x1) */
static axes_t face_axes(int dim) {
  axes_t a;
  int ivx = OG_IPR - dim;
  a.x = ivx;
  a.y = OG_IVX + ((ivx - OG_IVX) + 1) % 3;
  a.z = OG_IVX + ((ivx - OG_IVX) + 2) % 3;
  return a;
}

/* riemann_kernels.h:56-194, hllc_impl for T = double, no face background,
 * no species (dry fraction 1) */
static void hllc_impl(double* flx, const double* wl, const double* wr,
                      double el, double er, double gammal, double gammar,
                      double cl, double cr, int dim, double* face_pressure) {
  double pl = wl[OG_IPR], pr = wr[OG_IPR];
  axes_t ax = face_axes(dim);
  int ivx = ax.x, ivy = ax.y, ivz = ax.z;

  el += 0.5 * wl[OG_IDN] *
        (SQR(wl[OG_IVX]) + SQR(wl[OG_IVY]) + SQR(wl[OG_IVZ]));
  er += 0.5 * wr[OG_IDN] *
        (SQR(wr[OG_IVX]) + SQR(wr[OG_IVY]) + SQR(wr[OG_IVZ]));

  double rhoa = 0.5 * (wl[OG_IDN] + wr[OG_IDN]);
  double ca = 0.5 * (cl + cr);
  double pmid =
      0.5 * (wl[OG_IPR] + wr[OG_IPR] + (wl[ivx] - wr[ivx]) * rhoa * ca);

  double shock_l = pmid / wl[OG_IPR] - 1.0;
  double shock_r = pmid / wr[OG_IPR] - 1.0;
  double ql = (pmid <= wl[OG_IPR])
                  ? 1.0
                  : sqrt(1.0 + (gammal + 1) / (2 * gammal) * shock_l);
  double qr = (pmid <= wr[OG_IPR])
                  ? 1.0
                  : sqrt(1.0 + (gammar + 1) / (2 * gammar) * shock_r);

  double al = wl[ivx] - cl * ql;
  double ar = wr[ivx] + cr * qr;
  double bp = ar > 0.0 ? ar : 1.0e-10;
  double bm = al < 0.0 ? al : -1.0e-10;

  double vxl = wl[ivx] - al;
  double vxr = wr[ivx] - ar;
  double tl = wl[OG_IPR] + vxl * wl[OG_IDN] * wl[ivx];
  double tr = wr[OG_IPR] + vxr * wr[OG_IDN] * wr[ivx];
  double ml = wl[OG_IDN] * vxl;
  double mr = -(wr[OG_IDN] * vxr);
  double am = (tl - tr) / (ml + mr);
  double cp = (ml * tr + mr * tl) / (ml + mr);
  cp = cp > 0.0 ? cp : 0.0;
  if (face_pressure) *face_pressure = cp;

  vxl = wl[ivx] - bm;
  vxr = wr[ivx] - bp;
  const double rdl = 1.0, rdr = 1.0;
  double fl[5], fr[5];
  fl[OG_IDN] = wl[OG_IDN] * vxl * rdl;
  fr[OG_IDN] = wr[OG_IDN] * vxr * rdr;
  fl[ivx] = wl[OG_IDN] * wl[ivx] * vxl + wl[OG_IPR];
  fr[ivx] = wr[OG_IDN] * wr[ivx] * vxr + wr[OG_IPR];
  fl[ivy] = wl[OG_IDN] * wl[ivy] * vxl;
  fr[ivy] = wr[OG_IDN] * wr[ivy] * vxr;
  fl[ivz] = wl[OG_IDN] * wl[ivz] * vxl;
  fr[ivz] = wr[OG_IDN] * wr[ivz] * vxr;
  fl[OG_IPR] = el * vxl + pl * wl[ivx];
  fr[OG_IPR] = er * vxr + pr * wr[ivx];

  double sl, sr, sm;
  if (am >= 0.0) {
    sl = am / (am - bm);
    sr = 0.0;
    sm = -bm / (am - bm);
  } else {
    sl = 0.0;
    sr = -am / (bp - am);
    sm = bp / (bp - am);
  }
  flx[OG_IDN] = sl * fl[OG_IDN] + sr * fr[OG_IDN];
  flx[ivx] = sl * fl[ivx] + sr * fr[ivx] + sm * cp;
  flx[ivy] = sl * fl[ivy] + sr * fr[ivy];
  flx[ivz] = sl * fl[ivz] + sr * fr[ivz];
  flx[OG_IPR] = sl * fl[OG_IPR] + sr * fr[OG_IPR] + sm * cp * am;
}

/* riemann_kernels.h:197-255, lmars_impl for T = double, no species */
static void lmars_impl(double* flx, const double* wl, const double* wr,
                       double hl, double hr, double gammal, double gammar,
                       int dim, double* face_pressure) {
  axes_t ax = face_axes(dim);
  int ivx = ax.x, ivy = ax.y, ivz = ax.z;
  double wli[5] = {wl[OG_IDN], wl[ivx], wl[ivy], wl[ivz], wl[OG_IPR]};
  double wri[5] = {wr[OG_IDN], wr[ivx], wr[ivy], wr[ivz], wr[OG_IPR]};

  hl += 0.5 * (SQR(wli[OG_IVX]) + SQR(wli[OG_IVY]) + SQR(wli[OG_IVZ])) +
        wli[OG_IPR] / wli[OG_IDN];
  hr += 0.5 * (SQR(wri[OG_IVX]) + SQR(wri[OG_IVY]) + SQR(wri[OG_IVZ])) +
        wri[OG_IPR] / wri[OG_IDN];

  double rhobar = 0.5 * (wli[OG_IDN] + wri[OG_IDN]);
  double gamma_bar = 0.5 * (gammal + gammar);
  double cbar =
      sqrt(0.5 * gamma_bar * (wli[OG_IPR] + wri[OG_IPR]) / rhobar);
  double pbar = 0.5 * (wli[OG_IPR] + wri[OG_IPR]) +
                0.5 * (rhobar * cbar) * (wli[OG_IVX] - wri[OG_IVX]);
  if (face_pressure) *face_pressure = pbar;
  double ubar = 0.5 * (wli[OG_IVX] + wri[OG_IVX]) +
                0.5 / (rhobar * cbar) * (wli[OG_IPR] - wri[OG_IPR]);
  const double rd = 1.0;
  if (ubar > 0) {
    flx[OG_IDN] = ubar * wli[OG_IDN] * rd;
    flx[ivx] = ubar * wli[OG_IDN] * wli[OG_IVX] + pbar;
    flx[ivy] = ubar * wli[OG_IDN] * wli[OG_IVY];
    flx[ivz] = ubar * wli[OG_IDN] * wli[OG_IVZ];
    flx[OG_IPR] = ubar * wli[OG_IDN] * hl;
  } else {
    flx[OG_IDN] = ubar * wri[OG_IDN] * rd;
    flx[ivx] = ubar * wri[OG_IDN] * wri[OG_IVX] + pbar;
    flx[ivy] = ubar * wri[OG_IDN] * wri[OG_IVY];
    flx[ivz] = ubar * wri[OG_IDN] * wri[OG_IVZ];
    flx[OG_IPR] = ubar * wri[OG_IDN] * hr;
  }
}

/* riemann.cpp:232-262, the EOS face pass of an ideal gas: e = p/(gamma-1)
 * (ideal_gas.cpp:101-103), gamma = gammad, c = sqrt(gamma p / rho)
 * (equation_of_state.cpp:240-243) */
void og_hllc_face(const double* wl, const double* wr, double gammad, int dim,
                  double* flx, double* face_pressure) {
  double el = wl[OG_IPR] / (gammad - 1);
  double er = wr[OG_IPR] / (gammad - 1);
  double cl = sqrt(gammad * wl[OG_IPR] / wl[OG_IDN]);
  double cr = sqrt(gammad * wr[OG_IPR] / wr[OG_IDN]);
  hllc_impl(flx, wl, wr, el, er, gammad, gammad, cl, cr, dim, face_pressure);
}

void og_lmars_face(const double* wl, const double* wr, double gammad, int dim,
                   double* flx, double* face_pressure) {
  double hl = wl[OG_IPR] / (gammad - 1) / wl[OG_IDN];
  double hr = wr[OG_IPR] / (gammad - 1) / wr[OG_IDN];
  lmars_impl(flx, wl, wr, hl, hr, gammad, gammad, dim, face_pressure);
}

/* ideal_gas_impl.h:16-35 (the metric raise is the identity in Cartesian) */
void og_cons2prim_cell(const double* u, double* w, double gammad, int s) {
  w[OG_IDN * s] = u[OG_IDN * s];
  w[OG_IVX * s] = u[OG_IVX * s] / w[OG_IDN * s];
  w[OG_IVY * s] = u[OG_IVY * s] / w[OG_IDN * s];
  w[OG_IVZ * s] = u[OG_IVZ * s] / w[OG_IDN * s];
  double ke = 0.5 * (w[OG_IVX * s] * u[OG_IVX * s] + w[OG_IVY * s] * u[OG_IVY * s] +
                     w[OG_IVZ * s] * u[OG_IVZ * s]);
  double ie = u[OG_IPR * s] - ke;
  w[OG_IPR * s] = (gammad - 1.) * ie;
}

/* ------------------------------------------------------------------ */
/* block operations                                                    */
/* ------------------------------------------------------------------ */
/* the monitor's riemann.pstar_clamp: an HLLC face whose contact pressure
 * was clamped to zero (src/riemann/riemann.cpp:330-339) */
static void count_clamp(const og_block* b, double cp) {
  if (b->monitor && cp <= 0.0) {
#pragma omp atomic
    b->monitor[0] += 1;
  }
}

void og_default_block(og_block* b) {
  memset(b, 0, sizeof(*b));
  b->nvar = 5;
  b->nc1 = b->nc2 = b->nc3 = 1;
  b->ng = 3;
  b->dx1 = b->dx2 = b->dx3 = 1.;
  b->gammad = 1.4;
  b->riemann = OG_HLLC;
  b->shock = 1;
  /* Shu-Osher SSP-RK3 */
  b->wght[0][0] = 1.;      b->wght[0][1] = 0.;      b->wght[0][2] = 1.;
  b->wght[1][0] = 3. / 4.; b->wght[1][1] = 1. / 4.; b->wght[1][2] = 1. / 4.;
  b->wght[2][0] = 1. / 3.; b->wght[2][1] = 2. / 3.; b->wght[2][2] = 2. / 3.;
  b->flux_cov = 1;
  b->wb_wall_clamp = 1;
}

static size_t ncell(const og_block* b) {
  return (size_t)b->nc1 * b->nc2 * b->nc3;
}

void og_cons2prim(const og_block* b, const double* u, double* w) {
  size_t n = ncell(b);
#pragma omp parallel for schedule(static) if (n > 4096)
  for (long c = 0; c < (long)n; ++c) og_cons2prim_cell(u + c, w + c, b->gammad, (int)n);
}

/* ideal_gas.cpp:53-70: mom = v rho; E = p/(g-1) + 0.5 sum(v m) */
void og_prim2cons(const og_block* b, const double* w, double* u) {
  size_t n = ncell(b);
  for (size_t c = 0; c < n; ++c) {
    double rho = w[OG_IDN * n + c];
    double m1 = w[OG_IVX * n + c] * rho, m2 = w[OG_IVY * n + c] * rho,
           m3 = w[OG_IVZ * n + c] * rho;
    u[OG_IDN * n + c] = rho;
    u[OG_IVX * n + c] = m1;
    u[OG_IVY * n + c] = m2;
    u[OG_IVZ * n + c] = m3;
    double ke = 0.5 * (w[OG_IVX * n + c] * m1 + w[OG_IVY * n + c] * m2 +
                       w[OG_IVZ * n + c] * m3);
    double ie = w[OG_IPR * n + c] / (b->gammad - 1);
    u[OG_IPR * n + c] = ie + ke;
  }
}

/* size along direction d (1 = x1) and the element stride */
static int dir_size(const og_block* b, int d) {
  return d == 1 ? b->nc1 : d == 2 ? b->nc2 : b->nc3;
}
static size_t dir_stride(const og_block* b, int d) {
  return d == 1 ? 1 : d == 2 ? (size_t)b->nc1 : (size_t)b->nc1 * b->nc2;
}

/* bc_func.cpp:10-70 on one face. side 0 = inner, 1 = outer. */
static void bc_face(const og_block* b, double* q, int d, int side, int kind,
                    int primitive) {
  int n = dir_size(b, d), ng = b->ng;
  if (n == 1 || kind == OG_BC_NONE) return;
  size_t s = dir_stride(b, d);
  int nvar = b->nvar;
  size_t nc = ncell(b);
  /* iterate every line along d */
  int n1 = b->nc1, n2 = b->nc2, n3 = b->nc3;
  int la = d == 1 ? n2 : n1, lb = d == 3 ? n2 : n3;
  int normal = OG_IPR - (4 - d); /* var[4 - dim] with dim = 4 - d */
  for (int v = 0; v < nvar; ++v)
    for (int bidx = 0; bidx < lb; ++bidx)
      for (int a = 0; a < la; ++a) {
        size_t base;
        if (d == 1) base = ((size_t)bidx * n2 + a) * n1;
        else if (d == 2) base = (size_t)bidx * n2 * n1 + a;
        else base = (size_t)bidx * n1 + a;
        double* line = q + v * nc + base;
        for (int g = 0; g < ng; ++g) {
          int dst = side ? n - ng + g : g, src;
          double sign = 1.;
          if (kind == OG_BC_REFLECTING) {
            src = side ? n - ng - 1 - g : 2 * ng - 1 - g;
            if (v == normal) sign = -1.;
          } else if (kind == OG_BC_PERIODIC) {
            src = side ? ng + g : n - 2 * ng + g;
          } else { /* extrapolation */
            src = side ? n - ng - 1 : ng;
          }
          double val = line[src * s];
          line[dst * s] = sign < 0 ? val * -1 : val;
        }
      }
  (void)primitive;
}

void og_apply_bc(const og_block* b, double* q, int primitive) {
  for (int f = 0; f < 6; ++f) bc_face(b, q, 1 + f / 2, f % 2, b->bc[f], primitive);
}

/* reconstruct.cpp:217-229 + recon_point: face states along one line.
 * line: n cells, stride s, variable v. Writes ltf[f] (ILT) and rtf[f] (IRT)
 * for every face f = 0..n-1 of the line. */
static void recon_line(const double* line, size_t s, int n, int use_weno,
                       int scale, double* ilt, double* irt) {
  int il = 3, iu = n - 3;
  double st[5];
  for (int f = il - 1; f <= iu; ++f) { /* IRT: cm, cells f-2..f+2 */
    for (int k = 0; k < 5; ++k) st[k] = line[(size_t)(f - 2 + k) * s];
    irt[f] = use_weno ? weno5_point(st, 1, g_weno5_cm, scale)
                      : poly5_point(st, 1, g_cp5_cm);
  }
  for (int f = il; f <= iu + 1 && f < n; ++f) { /* ILT: cp, cells f-3..f+1 */
    for (int k = 0; k < 5; ++k) st[k] = line[(size_t)(f - 3 + k) * s];
    ilt[f] = use_weno ? weno5_point(st, 1, g_weno5_cp, scale)
                      : poly5_point(st, 1, g_cp5_cp);
  }
  for (int f = 0; f < il; ++f) {
    irt[f] = irt[il];
    ilt[f] = ilt[il];
  }
  for (int f = iu + 1; f < n; ++f) {
    irt[f] = irt[iu];
    ilt[f] = ilt[iu];
  }
}

void og_flux(const og_block* b, const double* w, int d, double* flux) {
  build_tables();
  int n = dir_size(b, d);
  size_t s = dir_stride(b, d), nc = ncell(b);
  int n1 = b->nc1, n2 = b->nc2, n3 = b->nc3;
  int la = d == 1 ? n2 : n1, lb = d == 3 ? n2 : n3;
  int dim = 4 - d; /* tensor axis of the reference's riemann dim */
  long nlines = (long)la * lb;
#pragma omp parallel for schedule(static) if (nlines > 16)
  for (long ln = 0; ln < nlines; ++ln) {
    int a = (int)(ln % la), bidx = (int)(ln / la);
    size_t base;
    if (d == 1) base = ((size_t)bidx * n2 + a) * n1;
    else if (d == 2) base = (size_t)bidx * n2 * n1 + a;
    else base = (size_t)bidx * n1 + a;
    double* ilt = (double*)malloc(sizeof(double) * 5 * n);
    double* irt = (double*)malloc(sizeof(double) * 5 * n);
    for (int v = 0; v < 5; ++v) {
      int use_weno = b->shock || v == OG_IDN;
      recon_line(w + v * nc + base, s, n, use_weno, b->weno_scale, ilt + v * n,
                 irt + v * n);
    }
    for (int f = 0; f < n; ++f) {
      double wl[5], wr[5], fx[5];
      for (int v = 0; v < 5; ++v) {
        wl[v] = ilt[v * n + f];
        wr[v] = irt[v * n + f];
      }
      if (b->riemann == OG_HLLC) {
        double cp;
        og_hllc_face(wl, wr, b->gammad, dim, fx, &cp);
        /* the interior faces: f = ng..n-ng along the line, interior cells
         * across it */
        int ng = b->ng;
        int inner_a = la == 1 || (a >= ng && a < la - ng);
        int inner_b = lb == 1 || (bidx >= ng && bidx < lb - ng);
        if (inner_a && inner_b && f >= ng && f <= n - ng) count_clamp(b, cp);
      } else {
        og_lmars_face(wl, wr, b->gammad, dim, fx, NULL);
      }
      for (int v = 0; v < 5; ++v) flux[v * nc + base + f * s] = fx[v];
    }
    free(ilt);
    free(irt);
  }
}

/* ------------------------------------------------------------------ */
/* well-balanced x1 reference (src/hydro/hydro_ref_x1_impl.h:20-272,   */
/* src/recon/x1_reference.cpp:96-240), uniform x1 grid, one block     */
/* column with physical x1 boundaries                                 */
/* ------------------------------------------------------------------ */
/* exp for the scan anchor, the same operations as the CUDA kernel's sg_exp
 * (snapy_gb300/csrc/sg_device.cuh), so oracle and GPU agree bit for bit:
 * Cody-Waite reduction x = k ln2 + r with a split ln2, then the Taylor
 * series of exp(r) to r^16 in Horner form, scaled by 2^k (about 2 ulp; the
 * reference calls libm's exp here, an ulp-level difference) */
static double sg_exp(double x) {
  const double ln2_hi = 6.93147180369123816490e-01;
  const double ln2_lo = 1.90821492927058770002e-10;
  const double inv_ln2 = 1.44269504088896338700e+00;
  double k = rint(x * inv_ln2);
  double r = (x - k * ln2_hi) - k * ln2_lo;
  double p = 1.0 / 20922789888000.0;
  p = p * r + 1.0 / 1307674368000.0;
  p = p * r + 1.0 / 87178291200.0;
  p = p * r + 1.0 / 6227020800.0;
  p = p * r + 1.0 / 479001600.0;
  p = p * r + 1.0 / 39916800.0;
  p = p * r + 1.0 / 3628800.0;
  p = p * r + 1.0 / 362880.0;
  p = p * r + 1.0 / 40320.0;
  p = p * r + 1.0 / 5040.0;
  p = p * r + 1.0 / 720.0;
  p = p * r + 1.0 / 120.0;
  p = p * r + 1.0 / 24.0;
  p = p * r + 1.0 / 6.0;
  p = p * r + 0.5;
  p = p * r + 1.0;
  p = p * r + 1.0;
  return scalbn(p, (int)k);
}

double og_exp(double x) { return sg_exp(x); }

static double ref_face(const double* lo, const double* hi, int f, int nc1) {
  return f < nc1 ? lo[f] : hi[nc1 - 1];
}

static double wall_rop(double r0, double r1, double k) {
  double q = r0 / r1, qk = k == floor(k) ? q : pow(q, k);
  for (int n = 1; k == floor(k) && n < k; ++n) qk *= q;
  double e = r1 > r0 ? r0 * qk : r0 + k * (r0 - r1);
  return e > 0. ? e : r0;
}

static double rop_at(const double* w, size_t plane, int j) {
  return w[OG_IDN * plane + j] / w[OG_IPR * plane + j];
}

static double rop_smooth(const double* w, size_t plane, int i, int jlo,
                         int jhi, int ext_lo, int ext_hi) {
  if (!(ext_lo && i - 2 < jlo) && !(ext_hi && i + 2 > jhi))
    return rop_at(w, plane, i < jlo ? jlo : (i > jhi ? jhi : i));
  double v[5];
  for (int m = -2; m <= 2; ++m) {
    int j = i + m;
    if (j < jlo)
      v[m + 2] = ext_lo ? wall_rop(rop_at(w, plane, jlo),
                                   rop_at(w, plane, jlo + 1), (double)(jlo - j))
                        : rop_at(w, plane, jlo);
    else if (j > jhi)
      v[m + 2] = ext_hi ? wall_rop(rop_at(w, plane, jhi),
                                   rop_at(w, plane, jhi - 1), (double)(j - jhi))
                        : rop_at(w, plane, jhi);
    else
      v[m + 2] = rop_at(w, plane, j);
  }
  return (v[0] + 4. * v[1] + 6. * v[2] + 4. * v[3] + v[4]) / 16.;
}

void og_ref_column(const og_block* b, const double* w, size_t plane,
                   double* psf_lo, double* psf_hi, double* pref, double* dsf,
                   double* dref, double* dsf_lr) {
  build_tables();
  const int nc1 = b->nc1, iu = nc1 - 1 - b->ng, il = nc1 - 1 - iu;
  const double grav = -b->grav1; /* the downward magnitude */
  const double dx = b->dx1;
  const int phys_in = b->bc[0] != OG_BC_NONE, phys_out = b->bc[1] != OG_BC_NONE;
  const int wall_clamp = b->wb_wall_clamp;
  /* hydro_ref_x1_scan_impl: anchored half a cell above the top cell */
  double rho_top = w[OG_IDN * plane + iu], pres_top = w[OG_IPR * plane + iu];
  double rdt_top = pres_top / rho_top;
  double top_anchor = pres_top * sg_exp(-grav * 0.5 * dx / rdt_top);
  const double minp = 2.2250738585072014e-308; /* DBL_MIN */
  double face = top_anchor;
  for (int i = iu; i >= 0; --i) {
    double dp = grav * w[OG_IDN * plane + i] * dx;
    double lo = face + dp, hi = face;
    psf_lo[i] = lo > minp ? lo : minp;
    psf_hi[i] = hi > minp ? hi : minp;
    face = lo;
  }
  face = top_anchor;
  for (int i = iu + 1; i < nc1; ++i) {
    double dp = grav * w[OG_IDN * plane + i] * dx;
    double lo = face, hi = lo - dp;
    psf_lo[i] = lo > minp ? lo : minp;
    psf_hi[i] = hi > minp ? hi : minp;
    face = hi;
  }
  /* hydro_ref_x1_cell_impl, uniform grid */
  static const double w6[6] = {11. / 1440., -31. / 480., 401. / 720.,
                               401. / 720., -31. / 480., 11. / 1440.};
  static const double w6e[2][6] = {
      {95. / 288., 1427. / 1440., -133. / 240., 241. / 720., -173. / 1440.,
       3. / 160.},
      {-3. / 160., 637. / 1440., 511. / 720., -43. / 240., 77. / 1440.,
       -11. / 1440.}};
  int thin = (iu - il + 1) < 5, fits = iu >= 4;
  int jlo = (wall_clamp && phys_in) ? il : 0;
  int jhi = (wall_clamp && phys_out) ? iu : nc1 - 1;
  int ext_lo = wall_clamp && phys_in && il + 1 <= iu;
  int ext_hi = wall_clamp && phys_out && iu - 1 >= il;
  double rs_prev = 0.;
  for (int i = 0; i < nc1; ++i) {
    int wall_in = wall_clamp && phys_in && i >= il && i < il + 2;
    int wall_out = wall_clamp && phys_out && i > iu - 2 && i <= iu;
    int clamp_in = wall_in && fits && !(thin && phys_out);
    int clamp_out = wall_out && fits && !(thin && phys_in);
    double lo = psf_lo[i], hi = psf_hi[i];
    double cell_pref = 0.5 * (lo + hi);
    double lower = lo < hi ? lo : hi, upper = lo > hi ? lo : hi;
#define SIX(start, wt, rev)                                              \
  do {                                                                   \
    double value = 0.;                                                   \
    for (int m = 0; m < 6; ++m)                                          \
      value += (wt)[(rev) ? 5 - m : m] *                                 \
               ref_face(psf_lo, psf_hi, (start) + m, nc1);               \
    if (value >= lower && value <= upper) cell_pref = value;             \
  } while (0)
    if (i >= 2 && i < nc1 - 2 && !wall_in && !wall_out) SIX(i - 2, w6, 0);
    if (clamp_in) SIX(il, w6e[i - il], 0);
    if (clamp_out) {
      int s0 = iu + 1 - 5;
      SIX(s0, w6e[4 - (i - s0)], 1);
    }
    if (!phys_in && i < 2) SIX(0, w6e[i], 0);
    if (!phys_out && i >= nc1 - 2) SIX(nc1 - 5, w6e[4 - (i - (nc1 - 5))], 1);
#undef SIX
    pref[i] = cell_pref;
    double rs = rop_smooth(w, plane, i, jlo, jhi, ext_lo, ext_hi);
    double rf = rs;
    if (i > 0) rf = 0.5 * (rs_prev + rs);
    rs_prev = rs;
    dref[i] = cell_pref * rs;
    dsf[i] = lo * rf;
  }
  /* x1_reference.cpp:183-238: per-side face density from the cp5 row on
   * dref, guarded by the two cells' range; a reflecting wall face takes the
   * mean of its two sides */
  double* dl = dsf_lr;       /* ILT */
  double* dr = dsf_lr + nc1; /* IRT */
  for (int f = 0; f < nc1; ++f) dl[f] = dr[f] = dsf[f];
  if (nc1 >= 6) {
    int il5 = 3, iu5 = nc1 - 3;
    double lin_l[nc1], lin_r[nc1];
    for (int f = 0; f < nc1; ++f) lin_l[f] = lin_r[f] = dsf[f];
    for (int f = il5 - 1; f <= iu5; ++f) lin_r[f] = poly5_point(dref + f - 2, 1, g_cp5_cm);
    for (int f = il5; f <= iu5 + 1 && f < nc1; ++f)
      lin_l[f] = poly5_point(dref + f - 3, 1, g_cp5_cp);
    for (int f = il5 - 1; f <= iu5 + 1; ++f) {
      double a = dref[f - 1], c = dref[f];
      double lo = a < c ? a : c, hi = a > c ? a : c;
      if (lin_l[f] >= lo && lin_l[f] <= hi) dl[f] = lin_l[f];
      if (lin_r[f] >= lo && lin_r[f] <= hi) dr[f] = lin_r[f];
    }
    for (int side = 0; side < 2; ++side) {
      if (b->bc[side] != OG_BC_REFLECTING) continue;
      int f = side == 0 ? il : iu + 1;
      double mean = 0.5 * (dl[f] + dr[f]);
      dl[f] = dr[f] = mean;
    }
  }
}

/* ------------------------------------------------------------------ */
/* the hydro tendency (src/hydro/hydro_forward.cpp:299-1235)           */
/* ------------------------------------------------------------------ */
static double recon_one(const double* c, size_t s, int weno, int side,
                        int scale) {
  double st[5];
  for (int k = 0; k < 5; ++k) st[k] = c[(ptrdiff_t)k * (ptrdiff_t)s];
  if (weno) return weno5_point(st, 1, side ? g_weno5_cp : g_weno5_cm, scale);
  return poly5_point(st, 1, side ? g_cp5_cp : g_cp5_cm);
}

/* face f states of a line (cell stride s, variable stride plane):
 * ILT from cells f-3..f+1 (cp), IRT from cells f-2..f+2 (cm) */
static void face_lr(const og_block* b, const double* line, size_t s,
                    size_t plane, int f, double* wl, double* wr) {
  for (int v = 0; v < 5; ++v) {
    int weno = b->shock || v == OG_IDN;
    const double* q = line + v * plane;
    wl[v] = recon_one(q + (ptrdiff_t)(f - 3) * (ptrdiff_t)s, s, weno, 1,
                      b->weno_scale);
    wr[v] = recon_one(q + (ptrdiff_t)(f - 2) * (ptrdiff_t)s, s, weno, 0,
                      b->weno_scale);
  }
}

static void riemann_face(const og_block* b, const double* wl, const double* wr,
                         int d, double* fx) {
  if (b->riemann == OG_HLLC) {
    double cp;
    og_hllc_face(wl, wr, b->gammad, 4 - d, fx, &cp);
    count_clamp(b, cp);
  } else {
    og_lmars_face(wl, wr, b->gammad, 4 - d, fx, NULL);
  }
}

#define CELL(v, j, i) ((size_t)(v) * nc + (size_t)(j) * n1 + (size_t)(i))

/* the tendency of one x2-x1 plane (the whole block when it is 2-D): w and
 * du point at the plane's first cell, variables `ncell(b)` apart; f3 (3-D
 * only) at the plane's x3 face fluxes, the next plane's face n1 n2 further,
 * added to the divergence after x1 and x2 as CoordinateImpl::divergence does
 * (src/coord/coordinate.cpp:618-662) */
/* t1, t2 (optional): the plane's register totals T_1, T_2 on the faces of
 * the interior cells, as the divergence reads them */
/* 3-D viscosity's parts of a plane (NULL otherwise): the velocity
 * divergence over the interior extended by one cell in every direction,
 * and the x3 faces' viscous fluxes (5 rows), both at the plane's first
 * cell like w */
typedef struct {
  const double* divv;
  const double* vf3;
} og_visc3;

static void tendency_plane(const og_block* b, const double* w, double dt,
                           double* du, const double* f3, double* t1,
                           double* t2, const og_visc3* v3) {
  const int n1 = b->nc1, n2 = b->nc2, ng = b->ng;
  const size_t nc = ncell(b);
  const int has2 = n2 > 1;
  const int il = ng, iu1 = n1 - ng; /* interior x1 cells il..iu1-1 */
  const int jl = has2 ? ng : 0, ju1 = has2 ? n2 - ng : 1;
  const int wb = b->grav1 != 0.;
  double* f1 = (double*)calloc(5 * nc, sizeof(double));
  double* f2 = has2 ? (double*)calloc(5 * nc, sizeof(double)) : NULL;

  /* (2) x1 faces il..iu1 of every interior column j */
#pragma omp parallel for schedule(static)
  for (int j = jl; j < ju1; ++j) {
    const double* col = w + (size_t)j * n1;
    double wl[5], wr[5], fx[5];
    if (!wb) {
      for (int f = il; f <= iu1; ++f) {
        face_lr(b, col, 1, nc, f, wl, wr);
        riemann_face(b, wl, wr, 1, fx);
        for (int v = 0; v < 5; ++v) f1[CELL(v, j, f)] = fx[v];
      }
    } else {
      double psf_lo[n1], psf_hi[n1], pref[n1], dsf[n1], dref[n1], dlr[2 * n1];
      og_ref_column(b, col, nc, psf_lo, psf_hi, pref, dsf, dref, dlr);
      /* WellBalancedX1::forward: the perturbations of p and rho about the
       * reference, even-mirrored into the wall ghosts */
      double wx[5 * n1];
      for (int v = 0; v < 5; ++v)
        for (int i = 0; i < n1; ++i) wx[v * n1 + i] = col[v * nc + i];
      for (int i = 0; i < n1; ++i) {
        wx[OG_IPR * n1 + i] -= pref[i];
        wx[OG_IDN * n1 + i] -= dref[i];
      }
      for (int c = 0; c < 2; ++c) {
        int v = c ? OG_IDN : OG_IPR;
        if (b->bc[0] != OG_BC_NONE)
          for (int g = 0; g < ng; ++g) wx[v * n1 + g] = wx[v * n1 + 2 * ng - 1 - g];
        if (b->bc[1] != OG_BC_NONE)
          for (int g = 0; g < ng; ++g)
            wx[v * n1 + iu1 + g] = wx[v * n1 + iu1 - 1 - g];
      }
      for (int f = il; f <= iu1; ++f) {
        face_lr(b, wx, 1, n1, f, wl, wr);
        double pl = wl[OG_IPR] + psf_lo[f], pr = wr[OG_IPR] + psf_lo[f];
        wl[OG_IPR] = pl > 0. ? pl : psf_lo[f];
        wr[OG_IPR] = pr > 0. ? pr : psf_lo[f];
        double dl = wl[OG_IDN] + dlr[f], dr = wr[OG_IDN] + dlr[n1 + f];
        double below = col[OG_IDN * nc + (f > 0 ? f - 1 : 0)];
        wl[OG_IDN] = dl > 0. ? dl : below;
        wr[OG_IDN] = dr > 0. ? dr : col[OG_IDN * nc + f];
        riemann_face(b, wl, wr, 1, fx);
        for (int v = 0; v < 5; ++v) f1[CELL(v, j, f)] = fx[v];
      }
    }
    /* boundary.prescribed: rows IDN and IPR on the x1 wall faces */
    if (b->bc[0] == OG_BC_REFLECTING) f1[CELL(OG_IDN, j, il)] = f1[CELL(OG_IPR, j, il)] = 0.;
    if (b->bc[1] == OG_BC_REFLECTING) f1[CELL(OG_IDN, j, iu1)] = f1[CELL(OG_IPR, j, iu1)] = 0.;
  }

  /* (3-4) x2 faces jl..ju1 of the x1-interior cells, with the covariance
   * row of _flux_covariance (Cartesian: IPR only, x1 cells 1..n1-2) */
  if (has2) {
    const int cov = b->flux_cov && n1 >= 3;
#pragma omp parallel for schedule(static)
    for (int j = jl; j <= ju1; ++j) {
      double wl[5], wr[5], fx[5];
      double h[n1], un[n1], rho[n1];
      for (int i = 0; i < n1; ++i) {
        face_lr(b, w + i, n1, nc, j, wl, wr);
        if (cov) {
          double wb_[5];
          for (int v = 0; v < 5; ++v) wb_[v] = 0.5 * (wl[v] + wr[v]);
          double p = wb_[OG_IPR];
          double enth = p / (b->gammad - 1) + p;
          rho[i] = wb_[OG_IDN];
          h[i] = enth / rho[i];
          un[i] = wb_[OG_IVY];
        }
        if (i >= il && i < iu1) {
          riemann_face(b, wl, wr, 2, fx);
          for (int v = 0; v < 5; ++v) f2[CELL(v, j, i)] = fx[v];
        }
      }
      if (cov) {
        for (int i = il; i < iu1; ++i) {
          double dx1 = b->x1v[i + 1] - b->x1v[i - 1];
          double s2 = b->dx1 * b->dx1 / 12.;
          double s2rho = s2 * rho[i];
          double d1h = (h[i + 1] - h[i - 1]) / dx1;
          double dun = (un[i + 1] - un[i - 1]) / dx1;
          f2[CELL(OG_IPR, j, i)] += s2rho * d1h * dun;
        }
      }
      int wall = (j == jl && b->bc[2] == OG_BC_REFLECTING) ||
                 (j == ju1 && b->bc[3] == OG_BC_REFLECTING);
      if (wall)
        for (int i = il; i < iu1; ++i)
          f2[CELL(OG_IDN, j, i)] = f2[CELL(OG_IPR, j, i)] = 0.;
    }
  }

  /* viscous fluxes (src/forcing/diffusion.cpp:553-683, Cartesian, kinematic
   * nu_iso, no heat conduction): momentum rows separately (vf1, vf2),
   * the energy row posted into the totals */
  double *vf1 = NULL, *vf2 = NULL;
  if (b->nu_iso > 0.) {
    vf1 = (double*)calloc(5 * nc, sizeof(double));
    vf2 = has2 ? (double*)calloc(5 * nc, sizeof(double)) : NULL;
    double* divv = (double*)calloc(nc, sizeof(double));
    /* div of velocity on the interior extended by one cell in each active
     * direction */
    int ja = has2 ? jl - 1 : 0, jb = has2 ? ju1 + 1 : 1;
    for (int j = ja; j < jb; ++j)
      for (int i = il - 1; i < iu1 + 1; ++i) {
        if (v3) { /* 3-D: the whole divergence, x3 term included */
          divv[(size_t)j * n1 + i] = v3->divv[(size_t)j * n1 + i];
          continue;
        }
        double dv = divv[(size_t)j * n1 + i];
        dv += (w[CELL(OG_IVX, j, i + 1)] - w[CELL(OG_IVX, j, i - 1)]) / (2. * b->dx1);
        if (has2)
          dv += (w[CELL(OG_IVY, j + 1, i)] - w[CELL(OG_IVY, j - 1, i)]) / (2. * b->dx2);
        divv[(size_t)j * n1 + i] = dv;
      }
    const size_t pl = (size_t)n1 * n2; /* the next x3 plane */
    const double nu = b->nu_iso;
    /* x1 faces f = il..iu1, x2 cells jl..ju1-1 */
    int wall_lo = b->bc[0] == OG_BC_REFLECTING, wall_hi = b->bc[1] == OG_BC_REFLECTING;
    int nface1 = iu1 + 1 - il;
    for (int j = jl; j < ju1; ++j)
      for (int f = il; f <= iu1; ++f) {
        double rf = 0.5 * (w[CELL(OG_IDN, j, f)] + w[CELL(OG_IDN, j, f - 1)]);
        if (nface1 >= 3) {
          double t = b->dx1 / (b->dx1 + b->dx1);
          if (f == il && wall_lo) {
            double vn = w[CELL(OG_IDN, j, il)], vx = w[CELL(OG_IDN, j, il + 1)];
            double wall = (1. + t) * vn - t * vx;
            rf = wall > 0. ? wall : vn;
          }
          if (f == iu1 && wall_hi) {
            double vn = w[CELL(OG_IDN, j, iu1 - 1)], vx = w[CELL(OG_IDN, j, iu1 - 2)];
            double wall = (1. + t) * vn - t * vx;
            rf = wall > 0. ? wall : vn;
          }
        }
        double divf = 0.5 * (divv[(size_t)j * n1 + f] + divv[(size_t)j * n1 + f - 1]);
        double e = 0.;
        for (int ivar = 0; ivar < 3; ++ivar) {
          int v = OG_IVX + ivar;
          double stress = (w[CELL(v, j, f)] - w[CELL(v, j, f - 1)]) / b->dx1;
          if (ivar == 0) {
            stress = 2. * stress - (2. / 3.) * divf;
          } else if (ivar == 1 && has2) {
            double below = (w[CELL(OG_IVX, j + 1, f - 1)] - w[CELL(OG_IVX, j - 1, f - 1)]) / (2. * b->dx2);
            double above = (w[CELL(OG_IVX, j + 1, f)] - w[CELL(OG_IVX, j - 1, f)]) / (2. * b->dx2);
            stress += 0.5 * (above + below);
          } else if (ivar == 2 && v3) {
            double below = (w[CELL(OG_IVX, j, f - 1) + pl] - w[CELL(OG_IVX, j, f - 1) - pl]) / (2. * b->dx3);
            double above = (w[CELL(OG_IVX, j, f) + pl] - w[CELL(OG_IVX, j, f) - pl]) / (2. * b->dx3);
            stress += 0.5 * (above + below);
          }
          double mf = -nu * rf * stress;
          vf1[CELL(v, j, f)] = mf;
          e += 0.5 * (w[CELL(v, j, f)] + w[CELL(v, j, f - 1)]) * mf;
        }
        vf1[CELL(OG_IPR, j, f)] = e;
      }
    /* x2 faces j = jl..ju1, x1 cells il..iu1-1 */
    if (has2)
      for (int j = jl; j <= ju1; ++j)
        for (int i = il; i < iu1; ++i) {
          double rf = 0.5 * (w[CELL(OG_IDN, j, i)] + w[CELL(OG_IDN, j - 1, i)]);
          double divf = 0.5 * (divv[(size_t)j * n1 + i] + divv[(size_t)(j - 1) * n1 + i]);
          double e = 0.;
          for (int ivar = 0; ivar < 3; ++ivar) {
            int v = OG_IVX + ivar;
            double stress = (w[CELL(v, j, i)] - w[CELL(v, j - 1, i)]) / b->dx2;
            if (ivar == 1) {
              stress = 2. * stress - (2. / 3.) * divf;
            } else if (ivar == 0) {
              double below = (w[CELL(OG_IVY, j - 1, i + 1)] - w[CELL(OG_IVY, j - 1, i - 1)]) / (2. * b->dx1);
              double above = (w[CELL(OG_IVY, j, i + 1)] - w[CELL(OG_IVY, j, i - 1)]) / (2. * b->dx1);
              stress += 0.5 * (above + below);
            } else if (ivar == 2 && v3) {
              double below = (w[CELL(OG_IVY, j - 1, i) + pl] - w[CELL(OG_IVY, j - 1, i) - pl]) / (2. * b->dx3);
              double above = (w[CELL(OG_IVY, j, i) + pl] - w[CELL(OG_IVY, j, i) - pl]) / (2. * b->dx3);
              stress += 0.5 * (above + below);
            }
            double mf = -nu * rf * stress;
            vf2[CELL(v, j, i)] = mf;
            e += 0.5 * (w[CELL(v, j, i)] + w[CELL(v, j - 1, i)]) * mf;
          }
          vf2[CELL(OG_IPR, j, i)] = e;
        }
    free(divv);
    /* post_fluxes: the energy rows join the totals; boundary.prescribed
     * again on the wall faces */
    for (int j = jl; j < ju1; ++j) {
      for (int f = il; f <= iu1; ++f) f1[CELL(OG_IPR, j, f)] += vf1[CELL(OG_IPR, j, f)];
      if (b->bc[0] == OG_BC_REFLECTING) f1[CELL(OG_IDN, j, il)] = f1[CELL(OG_IPR, j, il)] = 0.;
      if (b->bc[1] == OG_BC_REFLECTING) f1[CELL(OG_IDN, j, iu1)] = f1[CELL(OG_IPR, j, iu1)] = 0.;
    }
    if (has2)
      for (int j = jl; j <= ju1; ++j) {
        for (int i = il; i < iu1; ++i) f2[CELL(OG_IPR, j, i)] += vf2[CELL(OG_IPR, j, i)];
        int wall = (j == jl && b->bc[2] == OG_BC_REFLECTING) ||
                   (j == ju1 && b->bc[3] == OG_BC_REFLECTING);
        if (wall)
          for (int i = il; i < iu1; ++i) f2[CELL(OG_IDN, j, i)] = f2[CELL(OG_IPR, j, i)] = 0.;
      }
  }

  /* (5-6) divergence and du = -dt div on the interior */
  const double a1 = b->dx3 * b->dx2, a2 = b->dx3 * b->dx1;
  const double a3 = b->dx2 * b->dx1;
  const double vol = b->dx3 * (b->dx2 * b->dx1);
  const size_t plane = (size_t)n1 * n2;
  for (int v = 0; v < 5; ++v)
    for (size_t q = 0; q < plane; ++q) du[v * nc + q] = 0.;
  const double mdt = -dt;
  for (int v = 0; v < 5; ++v)
    for (int j = jl; j < ju1; ++j)
      for (int i = il; i < iu1; ++i) {
        size_t q = CELL(v, j, i);
        double dv = a1 * f1[q + 1] - a1 * f1[q];
        if (has2) dv = dv + (a2 * f2[q + n1] - a2 * f2[q]);
        if (f3) dv = dv + (a3 * f3[q + plane] - a3 * f3[q]);
        du[q] = mdt * (dv / vol);
      }

  /* constant gravity (src/forcing/const_gravity.cpp:37-42, nh = 1) */
  if (b->grav1 != 0.) {
    const double g = b->grav1, nh = 1.;
    for (int j = jl; j < ju1; ++j)
      for (int i = il; i < iu1; ++i) {
        double rho = w[CELL(OG_IDN, j, i)], vx = w[CELL(OG_IVX, j, i)];
        du[CELL(OG_IVX, j, i)] += dt * rho * g * nh;
        du[CELL(OG_IPR, j, i)] += dt * rho * vx * g * nh;
      }
  }

  /* the viscous momentum rows (DiffusionImpl::add): du -= dt div */
  if (vf1) {
    for (int v = 0; v < OG_IPR; ++v)
      for (int j = jl; j < ju1; ++j)
        for (int i = il; i < iu1; ++i) {
          size_t q = CELL(v, j, i);
          double dv = a1 * vf1[q + 1] - a1 * vf1[q];
          if (has2) dv = dv + (a2 * vf2[q + n1] - a2 * vf2[q]);
          if (v3) dv = dv + (a3 * v3->vf3[q + plane] - a3 * v3->vf3[q]);
          du[q] = du[q] - dt * (dv / vol);
        }
  }

  /* the x1 gravity energy correction (hydro_forward.cpp:1049-1124):
   * face-form work + corrected potential-energy work - the cell work */
  if (b->grav1 != 0.) {
    const double g = b->grav1;
    const int nx1 = iu1 - il;
    /* centroid slope stencil on x1v[il..iu1) (gravity_work.hpp:93-115) */
    double wt0[nx1], wt1[nx1], wt2[nx1];
    int i0[nx1];
    const double* x = b->x1v + il;
    if (nx1 >= 3) {
      double a = x[1] - x[0], bb = x[2] - x[1], c = x[nx1 - 2] - x[nx1 - 3],
             d = x[nx1 - 1] - x[nx1 - 2];
      for (int k = 0; k < nx1; ++k) {
        if (k == 0) {
          wt0[k] = -(2. * a + bb) / (a * (a + bb));
          wt1[k] = (a + bb) / (a * bb);
          wt2[k] = -(a / ((a + bb) * bb));
        } else if (k == nx1 - 1) {
          wt0[k] = d / (c * (c + d));
          wt1[k] = -((c + d) / (c * d));
          wt2[k] = (c + 2. * d) / ((c + d) * d);
        } else {
          double hm = x[k] - x[k - 1], hp = x[k + 1] - x[k];
          wt0[k] = -hp / (hm * (hm + hp));
          wt1[k] = (hp - hm) / (hm * hp);
          wt2[k] = hm / (hp * (hm + hp));
        }
        int jj = k < 1 ? 1 : (k > nx1 - 2 ? nx1 - 2 : k);
        i0[k] = jj - 1;
      }
    }
    for (int j = jl; j < ju1; ++j) {
      double drho[nx1];
      for (int k = 0; k < nx1; ++k) {
        int i = il + k;
        double vmd = (a1 * f1[CELL(OG_IDN, j, i + 1)] - a1 * f1[CELL(OG_IDN, j, i)]) / vol;
        drho[k] = mdt * vmd;
      }
      for (int k = 0; k < nx1; ++k) {
        int i = il + k;
        double hi = g * (b->x1f[i + 1] - b->x1v[i]);
        double lo = g * (b->x1f[i] - b->x1v[i]);
        double fm_hi = a1 * f1[CELL(OG_IDN, j, i + 1)], fm_lo = a1 * f1[CELL(OG_IDN, j, i)];
        double fgw = dt * ((hi * fm_hi - lo * fm_lo) / vol);
        if (nx1 >= 3) {
          double h = b->x1f[i + 1] - b->x1f[i];
          double gvar = g * (h * h / 12.);
          double sl = wt0[k] * drho[i0[k]];
          sl += wt1[k] * drho[i0[k] + 1];
          sl += wt2[k] * drho[i0[k] + 2];
          fgw += gvar * sl;
        }
        double rho = w[CELL(OG_IDN, j, i)], vx = w[CELL(OG_IVX, j, i)];
        double orig = dt * rho * vx * g * 1.;
        du[CELL(OG_IPR, j, i)] += fgw - orig;
      }
    }
  }
  if (t1)
    for (int v = 0; v < 5; ++v)
      for (int j = jl; j < ju1; ++j)
        for (int f = il; f <= iu1; ++f) t1[CELL(v, j, f)] = f1[CELL(v, j, f)];
  if (t2 && has2)
    for (int v = 0; v < 5; ++v)
      for (int j = jl; j <= ju1; ++j)
        for (int i = il; i < iu1; ++i) t2[CELL(v, j, i)] = f2[CELL(v, j, i)];
  free(f1);
  free(f2);
  free(vf1);
  free(vf2);
}

/* the covariance row of the x3 faces (HydroImpl::_flux_covariance with
 * dim 3, src/hydro/hydro_forward.cpp:58-231; Cartesian: the IPR row of the
 * x1-interior cells, sigma1^2 rho D1[h] D1[u_n] of the face means, added to
 * the face flux before the walls, :800-826) on the faces of the interior
 * (x2, x1) cells */
static void x3_covariance(const og_block* b, const double* w, double* f3) {
  const int n1 = b->nc1, n2 = b->nc2, n3 = b->nc3, ng = b->ng;
  if (!(b->flux_cov && n1 >= 3)) return;
  const size_t plane = (size_t)n1 * n2, nc = ncell(b);
  const int il = ng, iu1 = n1 - ng;
  const int jl = n2 > 1 ? ng : 0, ju1 = n2 > 1 ? n2 - ng : 1;
  const long nk = n3 - 2 * ng + 1, nj = ju1 - jl;
#pragma omp parallel for schedule(static)
  for (long q = 0; q < nk * nj; ++q) {
    const int k = ng + (int)(q / nj), j = jl + (int)(q % nj);
    double h[n1], un[n1], rho[n1];
    for (int i = il - 1; i <= iu1; ++i) {
      double wl[5], wr[5], wb_[5];
      face_lr(b, w + (size_t)j * n1 + i, plane, nc, k, wl, wr);
      for (int v = 0; v < 5; ++v) wb_[v] = 0.5 * (wl[v] + wr[v]);
      double p = wb_[OG_IPR];
      double enth = p / (b->gammad - 1) + p;
      rho[i] = wb_[OG_IDN];
      h[i] = enth / rho[i];
      un[i] = wb_[OG_IVZ];
    }
    for (int i = il; i < iu1; ++i) {
      double dx1 = b->x1v[i + 1] - b->x1v[i - 1];
      double s2 = b->dx1 * b->dx1 / 12.;
      double s2rho = s2 * rho[i];
      double d1h = (h[i + 1] - h[i - 1]) / dx1;
      double dun = (un[i + 1] - un[i - 1]) / dx1;
      f3[OG_IPR * nc + (size_t)k * plane + (size_t)j * n1 + i] += s2rho * d1h * dun;
    }
  }
}

/* 3-D viscosity (DiffusionImpl::cartesian_fluxes, src/forcing/
 * diffusion.cpp:553-683, kinematic nu_iso): the velocity divergence on the
 * interior extended by one cell in each direction (the x1, x2, x3 centred
 * derivatives summed in that order) and the x3 faces' viscous fluxes of the
 * interior (x2, x1) cells: rho the mean of the two cells, the stress of
 * each velocity component (the normal one 2 dv3/dx3 - 2/3 div v, the others
 * their x3 derivative plus the face mean of dv3/dx1, dv3/dx2), the momentum
 * rows -nu rho stress, the energy row the sum of each component's face mean
 * times its momentum row */
static void x3_viscosity(const og_block* b, const double* w, double** divv_out,
                         double** vf3_out) {
  const int n1 = b->nc1, n2 = b->nc2, n3 = b->nc3, ng = b->ng;
  const size_t nc = ncell(b), pl = (size_t)n1 * n2;
  const int has2 = n2 > 1;
  const int il = ng, iu1 = n1 - ng;
  const int jl = has2 ? ng : 0, ju1 = has2 ? n2 - ng : 1;
  double* divv = (double*)calloc(nc, sizeof(double));
  double* vf3 = (double*)calloc(5 * nc, sizeof(double));
#define W3(v, k, j, i) w[(size_t)(v) * nc + (size_t)(k) * pl + (size_t)(j) * n1 + (i)]
  const int ja = has2 ? jl - 1 : 0, jb = has2 ? ju1 + 1 : 1;
  for (int k = ng - 1; k <= n3 - ng; ++k)
    for (int j = ja; j < jb; ++j)
      for (int i = il - 1; i <= iu1; ++i) {
        double dv = 0.;
        dv += (W3(OG_IVX, k, j, i + 1) - W3(OG_IVX, k, j, i - 1)) / (2. * b->dx1);
        if (has2)
          dv += (W3(OG_IVY, k, j + 1, i) - W3(OG_IVY, k, j - 1, i)) / (2. * b->dx2);
        dv += (W3(OG_IVZ, k + 1, j, i) - W3(OG_IVZ, k - 1, j, i)) / (2. * b->dx3);
        divv[(size_t)k * pl + (size_t)j * n1 + i] = dv;
      }
  const double nu = b->nu_iso;
  for (int k = ng; k <= n3 - ng; ++k)
    for (int j = jl; j < ju1; ++j)
      for (int i = il; i < iu1; ++i) {
        const size_t c = (size_t)k * pl + (size_t)j * n1 + i;
        double rf = 0.5 * (W3(OG_IDN, k, j, i) + W3(OG_IDN, k - 1, j, i));
        double divf = 0.5 * (divv[c] + divv[c - pl]);
        double e = 0.;
        for (int ivar = 0; ivar < 3; ++ivar) {
          int v = OG_IVX + ivar;
          double stress = (W3(v, k, j, i) - W3(v, k - 1, j, i)) / b->dx3;
          if (ivar == 2) {
            stress = 2. * stress - (2. / 3.) * divf;
          } else if (ivar == 0) {
            double below = (W3(OG_IVZ, k - 1, j, i + 1) - W3(OG_IVZ, k - 1, j, i - 1)) / (2. * b->dx1);
            double above = (W3(OG_IVZ, k, j, i + 1) - W3(OG_IVZ, k, j, i - 1)) / (2. * b->dx1);
            stress += 0.5 * (above + below);
          } else if (has2) {
            double below = (W3(OG_IVZ, k - 1, j + 1, i) - W3(OG_IVZ, k - 1, j - 1, i)) / (2. * b->dx2);
            double above = (W3(OG_IVZ, k, j + 1, i) - W3(OG_IVZ, k, j - 1, i)) / (2. * b->dx2);
            stress += 0.5 * (above + below);
          }
          double mf = -nu * rf * stress;
          vf3[(size_t)v * nc + c] = mf;
          e += 0.5 * (W3(v, k, j, i) + W3(v, k - 1, j, i)) * mf;
        }
        vf3[(size_t)OG_IPR * nc + c] = e;
      }
#undef W3
  *divv_out = divv;
  *vf3_out = vf3;
}

/* the tendency, and the register totals T_d into T[d - 1] where set */
static void tendency_reg(const og_block* b, const double* w, double dt,
                         double* du, double* const* T) {
  build_tables();
  const size_t nc = ncell(b);
  if (b->nc3 == 1) {
    tendency_plane(b, w, dt, du, NULL, T[0], T[1], NULL);
    return;
  }
  /* 3-D (no viscosity): the x3 face fluxes of every line, the x3
   * covariance row, reflecting x3 walls prescribed, then each x2-x1 plane */
  const int n1 = b->nc1, n2 = b->nc2, n3 = b->nc3, ng = b->ng;
  const size_t plane = (size_t)n1 * n2;
  double* f3 = (double*)calloc(5 * nc, sizeof(double));
  og_flux(b, w, 3, f3);
  x3_covariance(b, w, f3);
  for (int side = 0; side < 2; ++side) {
    if (b->bc[4 + side] != OG_BC_REFLECTING) continue;
    int k = side ? n3 - ng : ng;
    for (size_t q = 0; q < plane; ++q)
      f3[OG_IDN * nc + k * plane + q] = f3[OG_IPR * nc + k * plane + q] = 0.;
  }
  double *divv3 = NULL, *vf3 = NULL;
  if (b->nu_iso > 0.) {
    x3_viscosity(b, w, &divv3, &vf3);
    /* post_fluxes: the x3 energy row joins the totals; the walls again */
    for (int k = ng; k <= n3 - ng; ++k)
      for (size_t q = 0; q < plane; ++q)
        f3[OG_IPR * nc + k * plane + q] += vf3[OG_IPR * nc + k * plane + q];
    for (int side = 0; side < 2; ++side) {
      if (b->bc[4 + side] != OG_BC_REFLECTING) continue;
      int k = side ? n3 - ng : ng;
      for (size_t q = 0; q < plane; ++q)
        f3[OG_IDN * nc + k * plane + q] = f3[OG_IPR * nc + k * plane + q] = 0.;
    }
  }
  memset(du, 0, sizeof(double) * 5 * nc);
  for (int k = ng; k < n3 - ng; ++k) {
    og_visc3 v3 = {divv3 ? divv3 + k * plane : NULL, vf3 ? vf3 + k * plane : NULL};
    tendency_plane(b, w + k * plane, dt, du + k * plane, f3 + k * plane,
                   T[0] ? T[0] + k * plane : NULL,
                   T[1] ? T[1] + k * plane : NULL, divv3 ? &v3 : NULL);
  }
  free(divv3);
  free(vf3);
  if (T[2]) {
    const int jl = n2 > 1 ? ng : 0, ju1 = n2 > 1 ? n2 - ng : 1;
    for (int v = 0; v < 5; ++v)
      for (int k = ng; k <= n3 - ng; ++k)
        for (int j = jl; j < ju1; ++j)
          for (int i = ng; i < n1 - ng; ++i) {
            size_t q = v * nc + k * plane + (size_t)j * n1 + i;
            T[2][q] = f3[q];
          }
  }
  free(f3);
}

void og_tendency(const og_block* b, const double* w, double dt, double* du) {
  double* none[3] = {NULL, NULL, NULL};
  tendency_reg(b, w, dt, du, none);
}

/* S_d <- w1 S_d + w2 dt T_d on the faces of the interior cells
 * (FluxRegister::end_stage, src/hydro/flux_register.cpp:761-776, its device
 * axpy src/utils/step_dt.cu:14-34: the add's alpha form, fused); stage 0
 * starts from S_d = 0 (begin_step) */
static void step_recursion(const og_block* b, int d, const double* T,
                           double* S, double w1, double w2dt, int first) {
  const int nc[3] = {b->nc1, b->nc2, b->nc3}, ng = b->ng;
  const size_t n = ncell(b);
  int lo[3], hi[3]; /* inclusive ranges of (i, j, k) */
  for (int a = 0; a < 3; ++a) {
    lo[a] = nc[a] > 1 ? ng : 0;
    hi[a] = nc[a] > 1 ? nc[a] - ng - 1 : 0;
  }
  hi[d - 1] += 1; /* the faces of the interior cells, both ends */
  for (int v = 0; v < 5; ++v)
    for (int k = lo[2]; k <= hi[2]; ++k)
      for (int j = lo[1]; j <= hi[1]; ++j)
        for (int i = lo[0]; i <= hi[0]; ++i) {
          size_t q = v * n + ((size_t)k * nc[1] + j) * nc[0] + i;
          S[q] = first ? fma(w2dt, T[q], 0.) : fma(w2dt, T[q], S[q] * w1);
        }
}
#undef CELL

/* the passive scalars' transport tendency ds = -dt div F_s
 * (ScalarImpl::forward, src/scalar/scalar.cpp:90-211, for the dry case with
 * neither limiter nor upper bound):
 *   - the face mixing ratio r = s_f / rho_f of each side, s_f and rho_f the
 *     scale-invariant reconstruction of the tracer density and of the total
 *     dry density of the stage input with the hydro's scheme for every row,
 *     floored at 0 (ReconstructImpl::forward without a hydro parent,
 *     src/recon/reconstruct.cpp:258-262), the donor cell's r where rho_f
 *     is not positive (scalar.cpp:100-104);
 *   - the upwind flux F_s = F_m r of the side F_m > 0 selects (the left
 *     state; else the right), F_m the hydro register's mass row of the face
 *     (riemann.cpp:164-170, scalar.cpp:106-121);
 *   - zero on the reflecting faces (boundary.prescribed, scalar.cpp:163-169);
 *   - the area-weighted divergence, as the hydro's.
 * fm[d - 1]: the mass flux along d (face f below cell f), or NULL */
/* the scalar face ratio of one side at face q along stride st
 * (ScalarImpl::forward's face_r, src/scalar/scalar.cpp:100-104): left (ILT,
 * cp over cells f-3..f+1, donor f-1) or right (IRT, cm over f-2..f+2, donor
 * f); s_f / rho_f of the floored scale-invariant WENO5 faces, or the donor
 * cell's ratio where rho_f is not positive */
static double scalar_face_r(const double* u, const double* sv, size_t nc,
                            size_t q, size_t st, int left) {
  const size_t c0 = q - (size_t)(left ? 3 : 2) * st;
  const size_t donor = left ? q - st : q;
  double rs[5], ss[5];
  for (int m = 0; m < 5; ++m) {
    rs[m] = u[OG_IDN * nc + c0 + m * st];
    ss[m] = sv[c0 + m * st];
  }
  double rf = weno5_point(rs, 1, left ? g_weno5_cp : g_weno5_cm, 1);
  if (rf < 0.) rf = 0.;
  double sf = weno5_point(ss, 1, left ? g_weno5_cp : g_weno5_cm, 1);
  if (sf < 0.) sf = 0.;
  return rf > 0. ? sf / rf : sv[donor] / u[OG_IDN * nc + donor];
}

/* the positivity limiter of the scalars (PositivityLimiter::apply with the
 * scalar's inputs, src/hydro/flux_positivity.cpp:29-268, no carry):
 *   theta_i = min(1, s_i V (1 - 4096 eps) / (dt out_i)), out_i the outgoing
 *   A F_s over the faces the divergence uses (1 where nothing drains);
 *   td the same of the dry density under the mass fluxes; phi = clamp(min
 *   of the neighbours' s / rho / its own, 0, 1) (0 where s / rho <= 0);
 *   theta <- theta + phi (min(theta / td, 1) - theta) where 0 < td < 1;
 *   the ghosts by the kScalar boundary functions; each face flux times its
 *   donor's theta (the lower cell where F_s > 0) */
static void scalar_limit(const og_block* b, const double* u, double* const* fm,
                         double dt, const double* s, double** fs) {
  const size_t nc = ncell(b);
  const int ns = b->nscalar, ng = b->ng;
  const int n[3] = {b->nc1, b->nc2, b->nc3};
  int lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    lo[a] = n[a] > 1 ? ng : 0;
    hi[a] = n[a] > 1 ? n[a] - ng - 1 : 0;
  }
  const double area[3] = {b->dx3 * b->dx2, b->dx3 * b->dx1, b->dx2 * b->dx1};
  const double vol = b->dx3 * (b->dx2 * b->dx1);
  const double margin = 4096. * DBL_EPSILON, tiny = DBL_MIN;
  /* channel 0..ns-1: the scalars; channel ns: the dry density */
  double* theta = (double*)malloc(sizeof(double) * (size_t)(ns + 1) * nc);
  for (int v = 0; v <= ns; ++v) {
    const double* f[3];
    for (int d = 0; d < 3; ++d)
      f[d] = fs[d] ? (v < ns ? fs[d] + (size_t)v * nc : fm[d]) : NULL;
    const double* q = v < ns ? s + (size_t)v * nc : u + OG_IDN * nc;
    double* th = theta + (size_t)v * nc;
    for (size_t c = 0; c < nc; ++c) th[c] = 1.;
    for (int k = lo[2]; k <= hi[2]; ++k)
      for (int j = lo[1]; j <= hi[1]; ++j)
        for (int i = lo[0]; i <= hi[0]; ++i) {
          const size_t c = ((size_t)k * n[1] + j) * n[0] + i;
          double out = 0.;
          for (int d = 0; d < 3; ++d) {
            if (!f[d]) continue;
            const size_t st = dir_stride(b, d + 1);
            const double up = area[d] * f[d][c + st], dn = area[d] * f[d][c];
            out = out + ((up > 0. ? up : 0.) + (-dn > 0. ? -dn : 0.));
          }
          const double avail = (q[c] > 0. ? q[c] : 0.) * vol * (1. - margin);
          const double drain = dt * out;
          if (drain > 0.) {
            const double t = avail / (drain > tiny ? drain : tiny);
            th[c] = t < 1. ? t : 1.;
          }
        }
  }
  const double* td = theta + (size_t)ns * nc;
  double* relaxed = (double*)malloc(sizeof(double) * (size_t)ns * nc);
  for (int v = 0; v < ns; ++v)
    for (size_t c = 0; c < nc; ++c) relaxed[(size_t)v * nc + c] = theta[(size_t)v * nc + c];
  for (int v = 0; v < ns; ++v)
    for (int k = lo[2]; k <= hi[2]; ++k)
      for (int j = lo[1]; j <= hi[1]; ++j)
        for (int i = lo[0]; i <= hi[0]; ++i) {
          const size_t c = ((size_t)k * n[1] + j) * n[0] + i;
          const double* sv = s + (size_t)v * nc;
          const double qc = sv[c] / u[OG_IDN * nc + c];
          double low = INFINITY;
          for (int d = 0; d < 3; ++d) {
            if (n[d] == 1 && d > 0) continue;
            const size_t st = dir_stride(b, d + 1);
            const double qm = sv[c - st] / u[OG_IDN * nc + c - st];
            const double qp = sv[c + st] / u[OG_IDN * nc + c + st];
            const double m = qm < qp ? qm : qp;
            low = d == 0 ? m : (m < low ? m : low);
          }
          double phi = 0.;
          if (qc > 0.) {
            phi = low / qc;
            phi = phi < 0. ? 0. : (phi > 1. ? 1. : phi);
          }
          const double t = theta[(size_t)v * nc + c], d0 = td[c];
          if (d0 < 1. && d0 > 0.) {
            const double r = t / d0;
            relaxed[(size_t)v * nc + c] = t + phi * ((r < 1. ? r : 1.) - t);
          }
        }
  og_scalar_bc(b, relaxed);
  for (int d = 0; d < 3; ++d) {
    if (!fs[d]) continue;
    const size_t st = dir_stride(b, d + 1);
    int flo[3], fhi[3];
    for (int a = 0; a < 3; ++a) {
      flo[a] = lo[a];
      fhi[a] = hi[a];
    }
    fhi[d] += 1;
    for (int v = 0; v < ns; ++v)
      for (int k = flo[2]; k <= fhi[2]; ++k)
        for (int j = flo[1]; j <= fhi[1]; ++j)
          for (int i = flo[0]; i <= fhi[0]; ++i) {
            const size_t c = ((size_t)k * n[1] + j) * n[0] + i;
            double* F = fs[d] + (size_t)v * nc + c;
            const double fac = *F > 0. ? relaxed[(size_t)v * nc + c - st]
                                       : relaxed[(size_t)v * nc + c];
            *F = *F * fac;
          }
  }
  free(relaxed);
  free(theta);
}

static void scalar_tendency(const og_block* b, const double* u,
                            const double* w, double* const* fm, double dt,
                            const double* s, double* ds) {
  const size_t nc = ncell(b);
  const int ns = b->nscalar, ng = b->ng;
  const int n[3] = {b->nc1, b->nc2, b->nc3};
  const int weno = 1; /* the hydro's scheme: weno5 for density rows */
  /* with the covariance row (x2 / x3 faces) the shared positivity limiter
   * runs too (scalar.cpp:145-160, 195-207) */
  const int cov_on = b->flux_cov && b->nc1 >= 3 && (b->nc2 > 1 || b->nc3 > 1);
  double* fs[3] = {NULL, NULL, NULL};
  int lo[3], hi[3]; /* interior cells, inclusive */
  for (int a = 0; a < 3; ++a) {
    lo[a] = n[a] > 1 ? ng : 0;
    hi[a] = n[a] > 1 ? n[a] - ng - 1 : 0;
  }
  for (int d = 1; d <= 3; ++d) {
    if (!fm[d - 1]) continue;
    fs[d - 1] = (double*)calloc((size_t)ns * nc, sizeof(double));
    const size_t st = dir_stride(b, d);
    int flo[3], fhi[3];
    for (int a = 0; a < 3; ++a) {
      flo[a] = lo[a];
      fhi[a] = hi[a];
    }
    fhi[d - 1] += 1; /* the faces of the interior cells, both ends */
    /* the covariance row of the x2 / x3 faces (scalar_flux_covariance,
     * src/hydro/hydro_forward.cpp:233-300, Cartesian, no species: q the
     * mean of the two sides' ratios, s2 rho D1[u_n] D1[q] with rho and u_n
     * of the hydro's face means) */
    const int cov = cov_on && d >= 2;
    const size_t xst = 1; /* x1 neighbours of a face */
    for (int k = flo[2]; k <= fhi[2]; ++k)
      for (int j = flo[1]; j <= fhi[1]; ++j)
        for (int i = flo[0]; i <= fhi[0]; ++i) {
          const size_t q = ((size_t)k * n[1] + j) * n[0] + i;
          const int f = d == 1 ? i : d == 2 ? j : k;
          const int wall = (f == ng && b->bc[2 * (d - 1)] == OG_BC_REFLECTING) ||
                           (f == n[d - 1] - ng &&
                            b->bc[2 * (d - 1) + 1] == OG_BC_REFLECTING);
          const double F = fm[d - 1][q];
          /* the side F > 0 selects */
          const int left = F > 0.;
          (void)weno;
          double un[3], rhof = 0.;
          if (cov)
            for (int m = -1; m <= 1; ++m) {
              double wl[5], wr[5];
              face_lr(b, w + q + m * (ptrdiff_t)xst - (size_t)f * st, st, nc, f,
                      wl, wr);
              un[m + 1] = 0.5 * (wl[d == 2 ? OG_IVY : OG_IVZ] +
                                 wr[d == 2 ? OG_IVY : OG_IVZ]);
              if (m == 0) rhof = 0.5 * (wl[OG_IDN] + wr[OG_IDN]);
            }
          for (int v = 0; v < ns; ++v) {
            const double* sv = s + (size_t)v * nc;
            const double r = scalar_face_r(u, sv, nc, q, st, left);
            double fl = F * r;
            if (cov) {
              double qf[3];
              for (int m = -1; m <= 1; ++m) {
                const size_t qm = q + m * (ptrdiff_t)xst;
                qf[m + 1] = 0.5 * (scalar_face_r(u, sv, nc, qm, st, 1) * 1. +
                                   scalar_face_r(u, sv, nc, qm, st, 0) * 1.);
              }
              const double dx1 = b->x1v[i + 1] - b->x1v[i - 1];
              const double s2 = b->dx1 * b->dx1 / 12.;
              const double d1u = (un[2] - un[0]) / dx1;
              const double d1q = (qf[2] - qf[0]) / dx1;
              fl = fl + s2 * rhof * d1u * d1q;
            }
            fs[d - 1][v * nc + q] = wall ? 0. : fl;
          }
        }
  }
  if (cov_on) scalar_limit(b, u, fm, dt, s, fs);
  const double a1 = b->dx3 * b->dx2, a2 = b->dx3 * b->dx1;
  const double a3 = b->dx2 * b->dx1;
  const double vol = b->dx3 * (b->dx2 * b->dx1);
  const double mdt = -dt;
  memset(ds, 0, sizeof(double) * ns * nc);
  for (int v = 0; v < ns; ++v)
    for (int k = lo[2]; k <= hi[2]; ++k)
      for (int j = lo[1]; j <= hi[1]; ++j)
        for (int i = lo[0]; i <= hi[0]; ++i) {
          const size_t q = v * nc + ((size_t)k * n[1] + j) * n[0] + i;
          double dv = 0.;
          if (fs[0]) dv = a1 * fs[0][q + 1] - a1 * fs[0][q];
          if (fs[1]) dv = dv + (a2 * fs[1][q + n[0]] - a2 * fs[1][q]);
          if (fs[2])
            dv = dv + (a3 * fs[2][q + (size_t)n[0] * n[1]] - a3 * fs[2][q]);
          ds[q] = mdt * (dv / vol);
        }
  for (int d = 0; d < 3; ++d) free(fs[d]);
}

/* kScalar boundary functions (bc_func.cpp:10-70): the hydro's, with no
 * sign flip */
void og_scalar_bc(const og_block* b, double* s) {
  og_block sb = *b;
  sb.nvar = b->nscalar;
  for (int f = 0; f < 6; ++f) {
    const int d = 1 + f / 2, side = f % 2, kind = b->bc[f];
    const int nd = dir_size(b, d), ng = b->ng;
    if (nd == 1 || kind == OG_BC_NONE) continue;
    const size_t st = dir_stride(b, d), nc = ncell(b);
    const int n1 = b->nc1, n2 = b->nc2, n3 = b->nc3;
    const int la = d == 1 ? n2 : n1, lb = d == 3 ? n2 : n3;
    for (int v = 0; v < sb.nvar; ++v)
      for (int bi = 0; bi < lb; ++bi)
        for (int a = 0; a < la; ++a) {
          size_t base;
          if (d == 1) base = ((size_t)bi * n2 + a) * n1;
          else if (d == 2) base = (size_t)bi * n2 * n1 + a;
          else base = (size_t)bi * n1 + a;
          double* line = s + v * nc + base;
          for (int g = 0; g < ng; ++g) {
            const int dst = side ? nd - ng + g : g;
            int src;
            if (kind == OG_BC_REFLECTING)
              src = side ? nd - ng - 1 - g : 2 * ng - 1 - g;
            else if (kind == OG_BC_PERIODIC)
              src = side ? ng + g : nd - 2 * ng + g;
            else
              src = side ? nd - ng - 1 : ng;
            line[dst * st] = line[src * st];
          }
        }
  }
}

/* the scalars' share of the implicit solve's dry transfer
 * (MeshBlockImpl::stage_advance, src/mesh/meshblock_advance.cpp:216-233): on
 * each x1 face the transfer q carries the donor's ratio r = s / rho of the
 * stage input (the cell below where q > 0), P = r q, capped by what the
 * donor holds after the explicit transport (donor_cap_cpu,
 * src/implicit/implicit_dispatch.cpp:54-70: along the column from the
 * bottom, q within [-held above, held below + the face below's P]), then
 * ds += (P - P_above) / V */
static void scalar_vic(const og_block* b, const double* u, const double* s,
                       const double* q, double* ds) {
  const int n1 = b->nc1, n2 = b->nc2, ng = b->ng, ns = b->nscalar;
  const size_t nc = ncell(b);
  const int il = ng, iu = n1 - ng - 1;
  const int jl = n2 > 1 ? ng : 0, ju1 = n2 > 1 ? n2 - ng : 1;
  const int n3 = b->nc3, kl = n3 > 1 ? ng : 0, ku1 = n3 > 1 ? n3 - ng : 1;
  const double vol = b->dx3 * (b->dx2 * b->dx1);
  double* P = (double*)malloc(sizeof(double) * (n1 + 1));
  for (int v = 0; v < ns; ++v)
    for (int k = kl; k < ku1; ++k)
    for (int j = jl; j < ju1; ++j) {
      const size_t c = ((size_t)k * n2 + j) * n1;
      const double* sv = s + v * nc + c;
      double* dv = ds + v * nc + c;
      const double* rho = u + OG_IDN * nc + c;
      const double* qc = q + c;
      for (int i = 0; i <= n1; ++i) P[i] = 0.;
      for (int i = il; i <= iu + 1; ++i) {
        const double M = qc[i];
        const double r = M > 0. ? sv[i - 1] / rho[i - 1] : sv[i] / rho[i];
        P[i] = r * M;
      }
      double avail = sv[il] + dv[il];
      avail = (avail < 0. ? 0. : avail) * vol;
      for (int i = il + 1; i <= iu; ++i) {
        double up = sv[i] + dv[i];
        up = (up < 0. ? 0. : up) * vol;
        double Q = P[i];
        if (Q > avail) Q = avail;
        if (Q < -up) Q = -up;
        P[i] = Q;
        avail = up + Q;
      }
      for (int i = il; i <= iu; ++i) dv[i] = dv[i] + (P[i] - P[i + 1]) / vol;
    }
  free(P);
}

void og_stage(const og_block* b, double* u, double* u0, double dt, int stage) {
#ifdef _OPENMP
  if (b->nthreads > 0) omp_set_num_threads(b->nthreads);
#endif
  size_t nc = ncell(b);
  size_t nall = nc * b->nvar;
  if (stage == 0) memcpy(u0, u, sizeof(double) * nall);
  double* w = (double*)malloc(sizeof(double) * nall);
  double* du = (double*)malloc(sizeof(double) * nall);
  og_cons2prim(b, u, w);
  /* the register totals where a step field or the totals are asked for */
  double* T[3] = {NULL, NULL, NULL};
  const int active[3] = {b->nc1 > 1, b->nc2 > 1, b->nc3 > 1};
  const int ns = b->scalar ? b->nscalar : 0;
  for (int d = 0; d < 3; ++d)
    if (active[d] && (b->step[d] || b->total[d] || ns > 0))
      T[d] = (double*)calloc(nall, sizeof(double));
  tendency_reg(b, w, dt, du, T);
  const double* wt = b->wght[stage];
  /* the scalars ride on the register's mass row before the implicit posts
   * enter T_1 (hydro_forward.cpp:918-922, scalar.cpp:106-116) */
  double* ds = NULL;
  if (ns > 0) {
    double* fm[3] = {NULL, NULL, NULL};
    for (int d = 0; d < 3; ++d)
      if (T[d]) fm[d] = T[d] + OG_IDN * nc;
    if (stage == 0) memcpy(b->scalar0, b->scalar, sizeof(double) * ns * nc);
    ds = (double*)malloc(sizeof(double) * ns * nc);
    scalar_tendency(b, u, w, fm, dt, b->scalar, ds);
  }
  /* the vertical implicit correction with dt_corr = wght2 dt
   * (hydro_forward.cpp:1153-1168); its posts enter T_1, whose wall faces
   * are prescribed again after it (hydro_forward.cpp:1195-1196) */
  double* vq = NULL;
  if (b->implicit_scheme == 9 || b->implicit_scheme == 1) {
    og_block bq = *b;
    if (ns > 0) bq.vic_q = vq = (double*)calloc(nc, sizeof(double));
    og_implicit_reg(&bq, w, wt[2] * dt, du, T[0], dt);
    if (ns > 0) scalar_vic(b, u, b->scalar, vq, ds);
    if (T[0]) {
      const int n1 = b->nc1, ng = b->ng;
      for (size_t r = 0; r < nc / n1; ++r)
        for (int side = 0; side < 2; ++side) {
          if (b->bc[side] != OG_BC_REFLECTING) continue;
          size_t q = r * n1 + (side ? n1 - ng : ng);
          T[0][OG_IDN * nc + q] = T[0][OG_IPR * nc + q] = 0.;
        }
    }
  }
  for (int d = 0; d < 3; ++d) {
    if (!T[d]) continue;
    if (b->step[d])
      step_recursion(b, d + 1, T[d], b->step[d], wt[1], wt[2] * dt, stage == 0);
    if (b->total[d]) memcpy(b->total[d], T[d], sizeof(double) * nall);
    free(T[d]);
  }
  /* the RK combine runs on every cell; du is zero outside the interior */
#pragma omp parallel for schedule(static) if (nall > 4096)
  for (long q = 0; q < (long)nall; ++q)
    u[q] = wt[0] * u0[q] + wt[1] * u[q] + wt[2] * du[q];
  og_apply_bc(b, u, 0);
  if (ns > 0) {
    double* s = b->scalar;
    for (size_t q = 0; q < (size_t)ns * nc; ++q)
      s[q] = wt[0] * b->scalar0[q] + wt[1] * s[q] + wt[2] * ds[q];
    og_scalar_bc(b, s);
    free(ds);
  }
  free(vq);
  free(w);
  free(du);
}

double og_max_dt(const og_block* b, const double* w) {
  size_t nc = ncell(b);
  double dtm[3] = {1e9, 1e9, 1e9};
  int ng = b->ng;
  int i0 = b->nc1 > 1 ? ng : 0, i1 = b->nc1 > 1 ? b->nc1 - ng : 1;
  int j0 = b->nc2 > 1 ? ng : 0, j1 = b->nc2 > 1 ? b->nc2 - ng : 1;
  int k0 = b->nc3 > 1 ? ng : 0, k1 = b->nc3 > 1 ? b->nc3 - ng : 1;
  double dx[3] = {b->dx1, b->dx2, b->dx3};
  int nn[3] = {b->nc1, b->nc2, b->nc3};
  for (int d = 0; d < 3; ++d) {
    if (nn[d] <= 1) continue;
    double best = INFINITY;
    for (int k = k0; k < k1; ++k)
      for (int j = j0; j < j1; ++j)
        for (int i = i0; i < i1; ++i) {
          size_t c = ((size_t)k * b->nc2 + j) * b->nc1 + i;
          double cs = sqrt(b->gammad * w[OG_IPR * nc + c] / w[OG_IDN * nc + c]);
          double v = dx[d] / (fabs(w[(OG_IVX + d) * nc + c]) + cs);
          /* an implicit x1 (scheme bit 0, more than a column) drops the x1
           * acoustic bound: dx1 / (|v1| cfl / advection_cfl) */
          if (d == 0 && (b->implicit_scheme & 1) && !(b->nc2 == 1 && b->nc3 == 1))
            v = dx[d] / (fabs(w[OG_IVX * nc + c]) * (b->cfl / 1.0));
          if (v < best) best = v;
        }
    dtm[d] = best;
  }
  double dt = dtm[0];
  if (dtm[1] < dt) dt = dtm[1];
  if (dtm[2] < dt) dt = dtm[2];
  /* sources.max_time_step: the viscous bound dx^2 / (2 ndim nu)
   * (src/forcing/diffusion.cpp:686-740) */
  if (b->nu_iso > 0.) {
    int ndim = 0;
    double dxm = 1.7976931348623157e308;
    for (int d = 0; d < 3; ++d)
      if (nn[d] > 1) {
        ++ndim;
        if (dx[d] < dxm) dxm = dx[d];
      }
    double dtv = dxm * dxm / (2. * ndim * b->nu_iso);
    if (dtv < dt) dt = dtv;
  }
  return dt;
}

void og_initialize(const og_block* b, double* w, double* u) {
  og_apply_bc(b, w, 1);
  og_prim2cons(b, w, u);
  og_apply_bc(b, u, 0);
}

/* ------------------------------------------------------------------ */
/* batched face helpers for the cubed-sphere oracle (numpy plumbing)  */
/* ------------------------------------------------------------------ */
/* n 5-cell stencils (row-major n x 5): weno5 (weno != 0) or cp5, side 1 the
 * cp row (the ILT state of the face above cell 2), 0 the cm row */
void og_recon_batch(const double* st, long n, int weno, int side, int scale,
                    double* out) {
  build_tables();
#pragma omp parallel for schedule(static) if (n > 4096)
  for (long q = 0; q < n; ++q)
    out[q] = weno ? og_weno5_face(st + 5 * q, side, scale)
                  : og_cp5_face(st + 5 * q, side);
}

/* shallow_roe_impl (src/riemann/riemann_kernels.h:447-495) with dir yz:
 * n faces, states wl, wr (n x 4: IDN = geopotential, IVX, IVY, IVZ), dim 2
 * (x2 faces: normal IVY) or 1 (x3 faces: normal IVZ) */
void og_shallow_roe_batch(const double* wl, const double* wr, long n, int dim,
                          double* flx) {
#pragma omp parallel for schedule(static) if (n > 4096)
  for (long q = 0; q < n; ++q) {
    const double* L = wl + 4 * q;
    const double* R = wr + 4 * q;
    double* F = flx + 4 * q;
    const int ivx = dim == 2 ? 2 : 3, ivy = dim == 2 ? 3 : 2, ivz = 1;
    double sqrtdl = sqrt(L[0]), sqrtdr = sqrt(R[0]);
    double isdlpdr = 1. / (sqrtdl + sqrtdr);
    double ubar = (L[ivx] * sqrtdl + R[ivx] * sqrtdr) * isdlpdr;
    double vbar = (L[ivy] * sqrtdl + R[ivy] * sqrtdr) * isdlpdr;
    double cbar = sqrt(0.5 * (L[0] + R[0]));
    double del0 = R[0] - L[0], delx = R[ivx] - L[ivx], dely = R[ivy] - L[ivy];
    double hbar = sqrt(L[0] * R[0]);
    double a1 = 0.5 * (cbar * del0 - hbar * delx) / cbar;
    double a2 = hbar * dely;
    double a3 = 0.5 * (cbar * del0 + hbar * delx) / cbar;
    double w0[4] = {0, 0, 0, 0}, w1[4] = {0, 0, 0, 0}, w2[4] = {0, 0, 0, 0};
    w0[0] = a1;
    w0[ivx] = a1 * (ubar - cbar);
    w0[ivy] = a1 * vbar;
    w1[ivy] = a2;
    w2[0] = a3;
    w2[ivx] = a3 * (ubar + cbar);
    w2[ivy] = a3 * vbar;
    double s0 = fabs(ubar - cbar), s1 = fabs(ubar), s2 = fabs(ubar + cbar);
    F[0] = 0.5 * (L[0] * L[ivx] + R[0] * R[ivx]);
    F[ivx] = 0.5 * (L[0] * L[ivx] * L[ivx] + 0.5 * L[0] * L[0] +
                    R[0] * R[ivx] * R[ivx] + 0.5 * R[0] * R[0]);
    F[ivy] = 0.5 * (L[0] * L[ivx] * L[ivy] + R[0] * R[ivx] * R[ivy]);
    F[ivz] = 0;
    for (int v = 0; v < 4; ++v)
      F[v] -= 0.5 * (s0 * w0[v] + s1 * w1[v] + s2 * w2[v]);
  }
}

/* HLLC for the shallow-water equations in geopotential form (Toro 2001,
 * Shock-Capturing Methods for Free-Surface Shallow Flows, ch. 10): wave
 * speeds S_L = min(u_L - c_L, u_R - c_R), S_R = max(u_L + c_L, u_R + c_R)
 * (c = sqrt(Phi)); the contact S* from the two HLL momentum states; HLL for
 * Phi and the normal momentum, the tangential momentum upwinded across S*.
 * The reference has no shallow-water HLLC; this is the checker of the
 * product's own.  Layout as og_shallow_roe_batch (dir yz). */
void og_hllc_sw_batch(const double* wl, const double* wr, long n, int dim,
                      double* flx) {
#pragma omp parallel for schedule(static) if (n > 4096)
  for (long q = 0; q < n; ++q) {
    const double* L = wl + 4 * q;
    const double* R = wr + 4 * q;
    double* F = flx + 4 * q;
    const int ivx = dim == 2 ? 2 : 3, ivy = dim == 2 ? 3 : 2, ivz = 1;
    const double cl = sqrt(L[0]), cr = sqrt(R[0]);
    const double ul = L[ivx], ur = R[ivx];
    const double sl = fmin(ul - cl, ur - cr), sr = fmax(ul + cl, ur + cr);
    const double ml = L[0] * ul, mr = R[0] * ur;
    const double fl0 = ml, fr0 = mr;
    const double fl1 = ml * ul + 0.5 * L[0] * L[0];
    const double fr1 = mr * ur + 0.5 * R[0] * R[0];
    double f0, f1, f2;
    if (sl >= 0.) {
      f0 = fl0;
      f1 = fl1;
      f2 = fl0 * L[ivy];
    } else if (sr <= 0.) {
      f0 = fr0;
      f1 = fr1;
      f2 = fr0 * R[ivy];
    } else {
      const double inv = 1. / (sr - sl);
      f0 = (sr * fl0 - sl * fr0 + sl * sr * (R[0] - L[0])) * inv;
      f1 = (sr * fl1 - sl * fr1 + sl * sr * (mr - ml)) * inv;
      const double den = R[0] * (ur - sr) - L[0] * (ul - sl);
      const double ss = (sl * R[0] * (ur - sr) - sr * L[0] * (ul - sl)) / den;
      f2 = ss >= 0. ? f0 * L[ivy] : f0 * R[ivy];
    }
    F[0] = f0;
    F[ivx] = f1;
    F[ivy] = f2;
    F[ivz] = 0.;
  }
}
