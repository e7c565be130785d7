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

#include <math.h>
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
      if (b->riemann == OG_HLLC)
        og_hllc_face(wl, wr, b->gammad, dim, fx, NULL);
      else
        og_lmars_face(wl, wr, b->gammad, dim, fx, NULL);
      for (int v = 0; v < 5; ++v) flux[v * nc + base + f * s] = fx[v];
    }
    free(ilt);
    free(irt);
  }
}

/* flux_register.cpp:700-740 with supply_prescribed (seam_register.cpp:184):
 * on a reflecting (wall) face plane the rows other than the momenta are
 * zeroed */
static void prescribe_walls(const og_block* b, double* flux, int d) {
  int n = dir_size(b, d);
  size_t s = dir_stride(b, d), nc = ncell(b);
  int n1 = b->nc1, n2 = b->nc2, n3 = b->nc3;
  int la = d == 1 ? n2 : n1, lb = d == 3 ? n2 : n3;
  for (int side = 0; side < 2; ++side) {
    if (b->bc[2 * (d - 1) + side] != OG_BC_REFLECTING) continue;
    int plane = side ? n - b->ng : b->ng;
    for (int bidx = 0; bidx < lb; ++bidx)
      for (int a = 0; a < la; ++a) {
        size_t base;
        if (d == 1) base = ((size_t)bidx * n2 + a) * n1;
        else if (d == 2) base = (size_t)bidx * n2 * n1 + a;
        else base = (size_t)bidx * n1 + a;
        flux[OG_IDN * nc + base + plane * s] = 0.;
        flux[OG_IPR * nc + base + plane * s] = 0.;
      }
  }
}

void og_stage(const og_block* b, double* u, double* u0, double dt, int stage) {
#ifdef _OPENMP
  if (b->nthreads > 0) omp_set_num_threads(b->nthreads);
#endif
  size_t nc = ncell(b);
  size_t nall = nc * b->nvar;
  if (stage == 0) memcpy(u0, u, sizeof(double) * nall);
  double* w = (double*)malloc(sizeof(double) * nall);
  double* f1 = (double*)calloc(nall, sizeof(double));
  double* f2 = b->nc2 > 1 ? (double*)calloc(nall, sizeof(double)) : NULL;
  double* f3 = b->nc3 > 1 ? (double*)calloc(nall, sizeof(double)) : NULL;
  og_cons2prim(b, u, w);
  if (b->nc1 > 1) {
    og_flux(b, w, 1, f1);
    prescribe_walls(b, f1, 1);
  }
  if (f2) {
    og_flux(b, w, 2, f2);
    prescribe_walls(b, f2, 2);
  }
  if (f3) {
    og_flux(b, w, 3, f3);
    prescribe_walls(b, f3, 3);
  }
  /* coordinate.cpp:488-515: area1 = dx3 dx2, area2 = dx3 dx1,
   * area3 = dx2 dx1, vol = dx3 (dx2 dx1) */
  double a1 = b->dx3 * b->dx2, a2 = b->dx3 * b->dx1, a3 = b->dx2 * b->dx1;
  double vol = b->dx3 * (b->dx2 * b->dx1);
  int ng = b->ng;
  int i0 = b->nc1 > 1 ? ng : 0, i1 = b->nc1 > 1 ? b->nc1 - ng : 1;
  int j0 = b->nc2 > 1 ? ng : 0, j1 = b->nc2 > 1 ? b->nc2 - ng : 1;
  int k0 = b->nc3 > 1 ? ng : 0, k1 = b->nc3 > 1 ? b->nc3 - ng : 1;
  const double* wt = b->wght[stage];
  double mdt = -dt;
  /* the RK combine runs on every cell; du is zero outside the interior */
#pragma omp parallel for schedule(static) if (nc > 4096)
  for (long c = 0; c < (long)nc; ++c) {
    int i = (int)(c % b->nc1), j = (int)((c / b->nc1) % b->nc2),
        k = (int)(c / ((size_t)b->nc1 * b->nc2));
    int inner = i >= i0 && i < i1 && j >= j0 && j < j1 && k >= k0 && k < k1;
    for (int v = 0; v < b->nvar; ++v) {
      size_t q = v * nc + c;
      double du = 0.;
      if (inner) {
        double dv = 0.;
        if (b->nc1 > 1) dv = dv + (a1 * f1[q + 1] - a1 * f1[q]);
        if (f2) dv = dv + (a2 * f2[q + b->nc1] - a2 * f2[q]);
        if (f3) dv = dv + (a3 * f3[q + (size_t)b->nc1 * b->nc2] - a3 * f3[q]);
        du = mdt * (dv / vol);
      }
      u[q] = wt[0] * u0[q] + wt[1] * u[q] + wt[2] * du;
    }
  }
  og_apply_bc(b, u, 0);
  free(w);
  free(f1);
  free(f2);
  free(f3);
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
          if (v < best) best = v;
        }
    dtm[d] = best;
  }
  double dt = dtm[0];
  if (dtm[1] < dt) dt = dtm[1];
  if (dtm[2] < dt) dt = dtm[2];
  return dt;
}

void og_initialize(const og_block* b, double* w, double* u) {
  og_apply_bc(b, w, 1);
  og_prim2cons(b, w, u);
  og_apply_bc(b, u, 0);
}
