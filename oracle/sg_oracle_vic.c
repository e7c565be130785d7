/*
 * CPU oracle, part 2: the vertical implicit correction (VIC) -- TEST
 * INFRASTRUCTURE ONLY.  FP64 restatement of the reference's block-
 * tridiagonal column solve on a Cartesian block without solids or species:
 * the full 5x5 blocks (implicit-scheme 9) and the partial 3x3 blocks of rows
 * and columns {rho, m1, E} (implicit-scheme 1: the tangential momenta folded
 * into the density column and the right-hand side, src/implicit/
 * vic_assemble_impl.h:152-214; the 3x3 forward sweep by the explicit inverse,
 * forward_sweep_impl.h:110-124; the donor transfer of the tangential momenta,
 * vic_redistribute_impl.h:178-200; their face posts,
 * implicit_hydro.cpp:520-530,662-666):
 *   src/implicit/implicit_hydro.cpp:301-560  ImplicitHydroImpl::forward_masked
 *   src/implicit/vic_assemble_impl.h:45-214  the blocks a, b, c of a cell
 *   src/implicit/flux_decomposition_impl.h   Roe average, eigenvectors, flux
 *                                            Jacobian
 *   src/implicit/vic_gravity_work_impl.h     the energy row's face work
 *   src/hydro/gravity_work.hpp:300-366       the corrected-PE rows K (bands,
 *                                            wall third points)
 *   src/implicit/forward_sweep_impl.h:30-131 block-Thomas forward sweep
 *   src/math/ludcmp.h, src/math/lubksb.h     scaled partial-pivot LU
 *   src/implicit/vic_kernels.h:100-160       back substitution, Woodbury
 *   src/implicit/vic_redistribute_impl.h     constituent column, cell map
 *   src/implicit/implicit_hydro.cpp:713-792  the gravity-work remainder
 * Matrix products are summed in index order (k = 0..4); the reference's
 * products go through Eigen, whose internal summation order is not restated
 * (an ulp-level difference, inside the 1e-12 parity bound).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "sg_oracle.h"

typedef double M5[5][5];
typedef double V5[5];

static void mat_mul(M5 out, M5 a, M5 b) {
  for (int r = 0; r < 5; ++r)
    for (int c = 0; c < 5; ++c) {
      double s = a[r][0] * b[0][c];
      for (int k = 1; k < 5; ++k) s += a[r][k] * b[k][c];
      out[r][c] = s;
    }
}

static void mat_vec(V5 out, M5 a, const double* v) {
  for (int r = 0; r < 5; ++r) {
    double s = a[r][0] * v[0];
    for (int k = 1; k < 5; ++k) s += a[r][k] * v[k];
    out[r] = s;
  }
}

/* flux_decomposition_impl.h: the x1 flux Jacobian of a cell (dir = 0) */
static void flux_jacobian(M5 J, double gm1, const double* w) {
  double v1 = w[1], v2 = w[2], v3 = w[3], rho = w[0], pres = w[4];
  double s2 = v1 * v1 + v2 * v2 + v3 * v3;
  double c1 = ((gm1 - 1) * s2 / 2 - (gm1 + 1) / gm1 * pres / rho) * v1;
  double c2 = (gm1 + 1) / gm1 * pres / rho + s2 / 2 - gm1 * v1 * v1;
  double m[5][5] = {
      {0, 1., 0., 0., 0.},
      {gm1 * s2 / 2 - v1 * v1, (2. - gm1) * v1, -gm1 * v2, -gm1 * v3, gm1},
      {-v1 * v2, v2, v1, 0., 0.},
      {-v1 * v3, v3, 0., v1, 0.},
      {c1, c2, -gm1 * v2 * v1, -gm1 * v3 * v1, (gm1 + 1) * v1}};
  memcpy(J, m, sizeof(m));
}

static void roe_average(double* prim, double gm1, const double* wl,
                        const double* wr) {
  double sqrtdl = sqrt(wl[0]), sqrtdr = sqrt(wr[0]);
  double isdlpdr = 1.0 / (sqrtdl + sqrtdr);
  prim[0] = sqrtdl * sqrtdr;
  prim[1] = (sqrtdl * wl[1] + sqrtdr * wr[1]) * isdlpdr;
  prim[2] = (sqrtdl * wl[2] + sqrtdr * wr[2]) * isdlpdr;
  prim[3] = (sqrtdl * wl[3] + sqrtdr * wr[3]) * isdlpdr;
  double el = wl[4] / gm1 + 0.5 * wl[0] * (wl[1] * wl[1] + wl[2] * wl[2] + wl[3] * wl[3]);
  double er = wr[4] / gm1 + 0.5 * wr[0] * (wr[1] * wr[1] + wr[2] * wr[2] + wr[3] * wr[3]);
  double hbar = ((el + wl[4]) / sqrtdl + (er + wr[4]) / sqrtdr) * isdlpdr;
  prim[4] = (hbar - 0.5 * (prim[1] * prim[1] + prim[2] * prim[2] + prim[3] * prim[3])) *
            gm1 / (gm1 + 1.) * prim[0];
}

/* |A| = R |Lambda| R^-1 at a face from its Roe average */
static void abs_jacobian(M5 A, double gm1, const double* wl, const double* wr) {
  double prim[5];
  roe_average(prim, gm1, wl, wr);
  double cs = sqrt(prim[4] * (gm1 + 1.) / prim[0]);
  double r = prim[0], u = prim[1], v = prim[2], w = prim[3], p = prim[4];
  double lam[5] = {fabs(u - cs), fabs(u), fabs(u + cs), fabs(u), fabs(u)};
  double ke = 0.5 * (u * u + v * v + w * w);
  double hp = (gm1 + 1.) / gm1 * p / r;
  double h = hp + ke;
  double R[5][5] = {{1., 1., 1., 0., 0.},
                    {u - cs, u, u + cs, 0., 0.},
                    {v, v, v, 1., 0.},
                    {w, w, w, 0., 1.},
                    {h - u * cs, ke, h + u * cs, v, w}};
  double Ri[5][5] = {
      {(cs * ke + u * hp) / (2. * cs * hp), (-hp - cs * u) / (2. * cs * hp),
       -v / (2. * hp), -w / (2. * hp), 1. / (2. * hp)},
      {(hp - ke) / hp, u / hp, v / hp, w / hp, -1. / hp},
      {(cs * ke - u * hp) / (2. * cs * hp), (hp - cs * u) / (2. * cs * hp),
       -v / (2. * hp), -w / (2. * hp), 1. / (2. * hp)},
      {-v, 0., 1., 0., 0.},
      {-w, 0., 0., 1., 0.}};
  M5 RL;
  for (int i = 0; i < 5; ++i)
    for (int k = 0; k < 5; ++k) RL[i][k] = R[i][k] * lam[k];
  mat_mul(A, RL, Ri);
}

/* ludcmp<double, 5, Implicit = true> (src/math/ludcmp.h) */
static int ludcmp5(M5 a, int* indx) {
  int i, imax = 0, j, k, d;
  double big, dum, sum, temp, vv[5], scale[5];
  const double tolerance = 8. * 5 * 2.220446049250313e-16;
  for (int r = 0; r < 5; ++r)
    for (int c = 0; c < 5; ++c)
      if (!isfinite(a[r][c])) return 0;
  d = 1;
  for (i = 0; i < 5; i++) {
    big = 0.0;
    for (j = 0; j < 5; j++)
      if ((temp = fabs(a[i][j])) > big) big = temp;
    if (big == 0.0) return 0;
    scale[i] = big;
    vv[i] = 1.0 / big;
    if (!isfinite(vv[i])) return 0;
  }
  for (j = 0; j < 5; j++) {
    for (i = 0; i < j; i++) {
      sum = a[i][j];
      for (k = 0; k < i; k++) sum -= a[i][k] * a[k][j];
      if (!isfinite(sum)) return 0;
      a[i][j] = sum;
    }
    big = 0.0;
    for (i = j; i < 5; i++) {
      sum = a[i][j];
      for (k = 0; k < j; k++) sum -= a[i][k] * a[k][j];
      if (!isfinite(sum)) return 0;
      a[i][j] = sum;
      dum = vv[i] * fabs(sum);
      if (!isfinite(dum)) return 0;
      if (dum >= big) {
        big = dum;
        imax = i;
      }
    }
    if (j != imax) {
      for (k = 0; k < 5; k++) {
        dum = a[imax][k];
        a[imax][k] = a[j][k];
        a[j][k] = dum;
      }
      d = -d;
      vv[imax] = vv[j];
      temp = scale[imax];
      scale[imax] = scale[j];
      scale[j] = temp;
    }
    indx[j] = imax;
    if (fabs(a[j][j]) / scale[j] <= tolerance) return 0;
    if (j != 4) {
      dum = (1.0 / a[j][j]);
      for (i = j + 1; i < 5; i++) a[i][j] *= dum;
    }
  }
  for (int r = 0; r < 5; ++r)
    for (int c = 0; c < 5; ++c)
      if (!isfinite(a[r][c])) return 0;
  return d;
}

/* lubksb with an M-column right-hand side (src/math/lubksb.h) */
static void lubksb5(M5 a, const int* indx, double b[5][8], int m) {
  for (int i = 0; i < 5; ++i) {
    int ip = indx[i];
    if (ip != i)
      for (int c = 0; c < m; ++c) {
        double t = b[ip][c];
        b[ip][c] = b[i][c];
        b[i][c] = t;
      }
    for (int j = 0; j < i; ++j)
      for (int c = 0; c < m; ++c) b[i][c] -= a[i][j] * b[j][c];
  }
  for (int i = 4; i >= 0; --i) {
    for (int j = i + 1; j < 5; ++j)
      for (int c = 0; c < m; ++c) b[i][c] -= a[i][j] * b[j][c];
    for (int c = 0; c < m; ++c) b[i][c] /= a[i][i];
  }
}

/* ludcmp<double, 3, Implicit = true> (src/math/ludcmp.h): the partial
 * matrix's sweep runs it only as the singularity screen */
static int ludcmp3(double a[3][3]) {
  int i, imax = 0, j, k, d;
  double big, dum, sum, temp, vv[3], scale[3];
  const double tolerance = 8. * 3 * 2.220446049250313e-16;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c)
      if (!isfinite(a[r][c])) return 0;
  d = 1;
  for (i = 0; i < 3; i++) {
    big = 0.0;
    for (j = 0; j < 3; j++)
      if ((temp = fabs(a[i][j])) > big) big = temp;
    if (big == 0.0) return 0;
    scale[i] = big;
    vv[i] = 1.0 / big;
    if (!isfinite(vv[i])) return 0;
  }
  for (j = 0; j < 3; j++) {
    for (i = 0; i < j; i++) {
      sum = a[i][j];
      for (k = 0; k < i; k++) sum -= a[i][k] * a[k][j];
      if (!isfinite(sum)) return 0;
      a[i][j] = sum;
    }
    big = 0.0;
    for (i = j; i < 3; i++) {
      sum = a[i][j];
      for (k = 0; k < j; k++) sum -= a[i][k] * a[k][j];
      if (!isfinite(sum)) return 0;
      a[i][j] = sum;
      dum = vv[i] * fabs(sum);
      if (!isfinite(dum)) return 0;
      if (dum >= big) {
        big = dum;
        imax = i;
      }
    }
    if (j != imax) {
      for (k = 0; k < 3; k++) {
        dum = a[imax][k];
        a[imax][k] = a[j][k];
        a[j][k] = dum;
      }
      d = -d;
      vv[imax] = vv[j];
      temp = scale[imax];
      scale[imax] = scale[j];
      scale[j] = temp;
    }
    if (fabs(a[j][j]) / scale[j] <= tolerance) return 0;
    if (j != 2) {
      dum = (1.0 / a[j][j]);
      for (i = j + 1; i < 3; i++) a[i][j] *= dum;
    }
  }
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c)
      if (!isfinite(a[r][c])) return 0;
  return d;
}

/* the inverse of a 3x3 block: the adjugate over the determinant, expanded
 * along column 0 (the reference inverts the block with Eigen's fixed-size
 * inverse, also a cofactor form; its order of operations is not restated) */
static void inverse3(double inv[3][3], double a[3][3]) {
  double c00 = a[1][1] * a[2][2] - a[1][2] * a[2][1];
  double c10 = a[0][2] * a[2][1] - a[0][1] * a[2][2];
  double c20 = a[0][1] * a[1][2] - a[0][2] * a[1][1];
  double det = a[0][0] * c00 + a[1][0] * c10 + a[2][0] * c20;
  double r = 1. / det;
  inv[0][0] = c00 * r;
  inv[0][1] = c10 * r;
  inv[0][2] = c20 * r;
  inv[1][0] = (a[1][2] * a[2][0] - a[1][0] * a[2][2]) * r;
  inv[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) * r;
  inv[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) * r;
  inv[2][0] = (a[1][0] * a[2][1] - a[1][1] * a[2][0]) * r;
  inv[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) * r;
  inv[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) * r;
}

static void mat3_mul(double out[3][3], double a[3][3], double b[3][3]) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      double s = a[r][0] * b[0][c];
      for (int k = 1; k < 3; ++k) s += a[r][k] * b[k][c];
      out[r][c] = s;
    }
}

static void mat3_vec(double out[3], double a[3][3], const double* v) {
  for (int r = 0; r < 3; ++r) {
    double s = a[r][0] * v[0];
    for (int k = 1; k < 3; ++k) s += a[r][k] * v[k];
    out[r] = s;
  }
}

/* the rows and columns {rho, m1, E} of the partial matrix */
static const int kRows3[3] = {0, 1, 4};

/* the corrected-PE slope stencil of n cells at centres x (gravity_work.hpp
 * :93-115): weights wt[3][n], first index i0[n] */
static void slope_stencil(const double* x, int n, double* wt0, double* wt1,
                          double* wt2, int* i0) {
  double a = x[1] - x[0], bb = x[2] - x[1], c = x[n - 2] - x[n - 3],
         d = x[n - 1] - x[n - 2];
  for (int k = 0; k < n; ++k) {
    if (k == 0) {
      wt0[k] = -(2. * a + bb) / (a * (a + bb));
      wt1[k] = (a + bb) / (a * bb);
      wt2[k] = -(a / ((a + bb) * bb));
    } else if (k == n - 1) {
      wt0[k] = d / (c * (c + d));
      wt1[k] = -((c + d) / (c * d));
      wt2[k] = (c + 2. * d) / ((c + d) * d);
    } else {
      double hm = x[k] - x[k - 1], hp = x[k + 1] - x[k];
      wt0[k] = -hp / (hm * (hm + hp));
      wt1[k] = (hp - hm) / (hm * hp);
      wt2[k] = hm / (hp * (hm + hp));
    }
    int jj = k < 1 ? 1 : (k > n - 2 ? n - 2 : k);
    i0[k] = jj - 1;
  }
}

/* the redistribution of a solved column: vic_constituent_column (no
 * species: the per-cell total-mass increments phi, the zero-sum face
 * transfers M by prefix sum, the donor-upwinded dry transfer q with the
 * sequential availability clamp), for the partial matrix
 * vic_tangential_momentum_column (each face's moved total mass carries the
 * donor cell's tangential velocity), then vic_redistribute_cell
 * (src/implicit/vic_redistribute_impl.h:60-232).  w, du: 5 rows with row
 * stride st; dl: the solution per layer (rows 0-4; the partial matrix's
 * tangential rows hold the explicit du); vol per layer.  mf_dn[n] zeroed,
 * mf_M[n + 1] and mf_q[n + 1] zeroed on entry. */
static void redistribute_column(int n, const double* w, size_t st, double* du,
                                V5* dl, const double* vol, int partial,
                                double* mf_dn, double* mf_M, double* mf_q) {
#define WV(v, i) w[(size_t)(v) * st + (i)]
#define DU(v, i) du[(size_t)(v) * st + (i)]
  double* phi = calloc(n, sizeof(double));
  double R = 0, S = 0;
  for (int i = 0; i < n; ++i) {
    double explicit_total = DU(0, i);
    phi[i] = (dl[i][0] - explicit_total) * vol[i];
    R += phi[i];
    S += WV(0, i) * vol[i];
  }
  double M = 0;
  for (int i = 0; i < n; ++i) {
    mf_M[i] = M;
    M -= phi[i] - R * (WV(0, i) * vol[i] / S);
  }
  double avail = (WV(0, 0) * 1. + DU(0, 0)) * vol[0];
  if (avail < 0) avail = 0;
  for (int i = 0; i + 1 < n; ++i) {
    double avail_up = (WV(0, i + 1) * 1. + DU(0, i + 1)) * vol[i + 1];
    if (avail_up < 0) avail_up = 0;
    double Mf = mf_M[i + 1];
    double q = Mf > 0 ? Mf * 1. : Mf * 1.;
    if (q > avail) q = avail;
    if (q < -avail_up) q = -avail_up;
    mf_dn[i] -= q / vol[i];
    mf_dn[i + 1] += q / vol[i + 1];
    mf_q[i + 1] = q;
    avail = avail_up + q;
  }
  for (int i = 0; i < n; ++i) {
    DU(0, i) += mf_dn[i];
    DU(1, i) = dl[i][1];
    DU(2, i) = dl[i][2];
    DU(3, i) = dl[i][3];
    DU(4, i) = dl[i][4];
  }
  if (partial)
    for (int i = 0; i + 1 < n; ++i) {
      double q = mf_q[i + 1];
      int donor = q > 0 ? i : i + 1;
      for (int t = 2; t < 4; ++t) {
        double pm = q * WV(t, donor);
        if (pm == 0) continue;
        DU(t, i) -= pm / vol[i];
        DU(t, i + 1) += pm / vol[i + 1];
      }
    }
  free(phi);
#undef WV
#undef DU
}

/* the redistribution alone, for the reference's own known-answer property
 * of the partial matrix (tests/test_backward_substitution.cpp:308-365):
 * n layers, w and du 5 x n (row stride n), vol[n], delta n x 3 (the 3x3
 * solution: total mass, m1, E) */
void og_vic_redistribute_partial(int n, const double* w, double* du,
                                 const double* vol, const double* delta) {
  V5* dl = malloc(sizeof(V5) * n);
  for (int i = 0; i < n; ++i) {
    dl[i][0] = delta[3 * i];
    dl[i][1] = delta[3 * i + 1];
    dl[i][2] = du[2 * (size_t)n + i];
    dl[i][3] = du[3 * (size_t)n + i];
    dl[i][4] = delta[3 * i + 2];
  }
  double* mf_dn = calloc(n, sizeof(double));
  double* mf_M = calloc(n + 1, sizeof(double));
  double* mf_q = calloc(n + 1, sizeof(double));
  redistribute_column(n, w, n, du, dl, vol, 1, mf_dn, mf_M, mf_q);
  free(dl);
  free(mf_dn);
  free(mf_M);
  free(mf_q);
}

/* one column: n interior layers; w, du (5 rows each) with row stride `st`
 * and cell stride 1, w readable at layers -1 and n (ghosts) */
/* t1 (optional): the column's x1 register totals at faces 0..n, strided by
 * st per variable; the solve posts its face transfers into them
 * (ImplicitHydroImpl::post_, src/implicit/implicit_hydro.cpp:625-673) with
 * kdt = dt A_f, the step's dt */
/* qout (optional): the column's clamped dry transfer q of faces 0..n
 * (MASS(IVY) of ImplicitHydroImpl's mass correction, zero on the walls and
 * for a failed column), for the scalars' share of it */
static int vic_column(const og_block* b, const double* w, size_t st, double* du,
                      int n, double dtc, const double* x1f, const double* x1v,
                      double* t1, double kdt, double* qout) {
  const double grav = b->grav1, gm1 = b->gammad - 1.;
  const double area = b->dx3 * b->dx2, vol = b->dx3 * (b->dx2 * b->dx1);
  M5* A = (M5*)malloc(sizeof(M5) * n);
  M5* B = (M5*)malloc(sizeof(M5) * n);
  M5* C = (M5*)malloc(sizeof(M5) * n);
  V5* dl = (V5*)malloc(sizeof(V5) * n);
  V5* z0 = (V5*)malloc(sizeof(V5) * n);
  V5* z1 = (V5*)malloc(sizeof(V5) * n);
  double* du0 = (double*)malloc(sizeof(double) * 5 * n);
  double *kmid = malloc(sizeof(double) * n), *klo = malloc(sizeof(double) * n),
         *khi = malloc(sizeof(double) * n), *gv = malloc(sizeof(double) * n);
  double *wt0 = malloc(sizeof(double) * n), *wt1 = malloc(sizeof(double) * n),
         *wt2 = malloc(sizeof(double) * n);
  int* i0 = malloc(sizeof(int) * n);
  /* the partial matrix (implicit-scheme 1: bit 3 of the scheme clear) */
  const int partial = !((b->implicit_scheme >> 3) & 1);
  typedef double M3[3][3];
  typedef double V3[3];
  M3* A3 = partial ? (M3*)malloc(sizeof(M3) * n) : NULL;
  M3* B3 = partial ? (M3*)malloc(sizeof(M3) * n) : NULL;
  M3* C3 = partial ? (M3*)malloc(sizeof(M3) * n) : NULL;
  V3* rc = partial ? (V3*)calloc(n, sizeof(V3)) : NULL; /* rhs_corr */
  V3* d3 = partial ? (V3*)malloc(sizeof(V3) * n) : NULL;
  V3* y0 = partial ? (V3*)malloc(sizeof(V3) * n) : NULL;
  V3* y1 = partial ? (V3*)malloc(sizeof(V3) * n) : NULL;
  int ok = 1;
#define WV(v, i) w[(size_t)(v) * st + (i)]
#define DU(v, i) du[(size_t)(v) * st + (i)]
  for (int v = 0; v < 5; ++v)
    for (int i = 0; i < n; ++i) du0[v * n + i] = DU(v, i);
  /* the input screen */
  for (int i = 0; i < n && ok; ++i)
    for (int v = 0; v < 5; ++v)
      if (!isfinite(DU(v, i)) || !isfinite(WV(v, i))) ok = 0;
  /* (1) assemble (vic_assemble_impl, N = 5, dir = 0) */
  for (int i = 0; i < n && ok; ++i) {
    double wl[5], wr[5], wn[5];
    for (int v = 0; v < 5; ++v) {
      wl[v] = WV(v, i - 1);
      wr[v] = WV(v, i);
      wn[v] = WV(v, i + 1);
    }
    M5 Jp, Jc, Jn, Am, Ap;
    flux_jacobian(Jp, gm1, wl);
    flux_jacobian(Jc, gm1, wr);
    abs_jacobian(Am, 0.5 * (b->gammad + b->gammad) - 1., wl, wr);
    flux_jacobian(Jn, gm1, wn);
    abs_jacobian(Ap, 0.5 * (b->gammad + b->gammad) - 1., wr, wn);
    double half_inv_vol = 0.5 / vol;
    double lower = 0.5 * area * (x1v[i] - x1f[i]) / vol;
    double upper = 0.5 * area * (x1f[i + 1] - x1v[i]) / vol;
    for (int r = 0; r < 5; ++r)
      for (int c = 0; c < 5; ++c) {
        double phi = (r == 1 && c == 0) || (r == 4 && c == 1) ? grav : 0.;
        A[i][r][c] = (Am[r][c] * area + Ap[r][c] * area + (area - area) * Jc[r][c]) *
                         half_inv_vol - phi;
        B[i][r][c] = -(Am[r][c] + Jp[r][c]) * area * half_inv_vol;
        C[i][r][c] = -(Ap[r][c] - Jn[r][c]) * area * half_inv_vol;
      }
    for (int r = 0; r < 5; ++r) A[i][r][r] += 1. / dtc;
    /* vic_gravity_work_rows: e = IPR, m = IVX */
    for (int k = 0; k < 5; ++k) {
      A[i][4][k] -= grav * (upper * Ap[0][k] - lower * Am[0][k]);
      B[i][4][k] -= grav * lower * Am[0][k];
      C[i][4][k] += grav * upper * Ap[0][k];
    }
    A[i][4][1] += grav * (1. - lower - upper);
    B[i][4][1] -= grav * lower;
    C[i][4][1] -= grav * upper;
    const double bnd[5] = {1., -1., 1., 1., 1.};
    if (i == 0)
      for (int r = 0; r < 5; ++r)
        for (int c = 0; c < 5; ++c) A[i][r][c] += B[i][r][c] * bnd[c];
    if (i == n - 1)
      for (int r = 0; r < 5; ++r)
        for (int c = 0; c < 5; ++c) A[i][r][c] += C[i][r][c] * bnd[c];
    if (partial) {
      /* the 3x3 blocks are the {rho, m1, E} rows and columns of the same
       * entries (each entry is the same expression); the m_t columns of
       * those rows (aT, bT, cT: columns IVY, IVZ with the same terms, the
       * energy row's face work and the wall mirror included) fold into the
       * density column at the cell's v_t and into the right-hand side at the
       * frozen remainder q_t = du[m_t] - v_t du[rho]
       * (vic_assemble_impl.h:167-213) */
      double aT[3][2], bT[3][2], cT[3][2];
      for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) {
          A3[i][r][c] = A[i][kRows3[r]][kRows3[c]];
          B3[i][r][c] = B[i][kRows3[r]][kRows3[c]];
          C3[i][r][c] = C[i][kRows3[r]][kRows3[c]];
        }
        for (int k = 0; k < 2; ++k) {
          aT[r][k] = A[i][kRows3[r]][2 + k];
          bT[r][k] = B[i][kRows3[r]][2 + k];
          cT[r][k] = C[i][kRows3[r]][2 + k];
        }
      }
      for (int r = 0; r < 3; ++r) rc[i][r] = 0.;
      for (int side = 0; side < 3; ++side) {
        int j = side == 0 ? i : (side == 1 ? i - 1 : i + 1);
        if (side == 1 && i == 0) continue;     /* merged lower wall */
        if (side == 2 && i == n - 1) continue; /* merged upper wall */
        double(*blk)[3] = side == 0 ? A3[i] : (side == 1 ? B3[i] : C3[i]);
        double(*tb)[2] = side == 0 ? aT : (side == 1 ? bT : cT);
        double drho = DU(0, j);
        for (int k = 0; k < 2; ++k) {
          double v = WV(2 + k, j);
          double q = DU(2 + k, j) - v * drho;
          if (v != 0)
            for (int r = 0; r < 3; ++r) blk[r][0] = blk[r][0] + tb[r][k] * v;
          if (q != 0)
            for (int r = 0; r < 3; ++r) rc[i][r] = rc[i][r] + tb[r][k] * q;
        }
      }
    }
  }
  /* (2) couple_radial_exact: the corrected-PE rows K in the (IPR, IDN)
   * entry of the blocks, and the explicit part moved to the right side */
  int wood = n >= 3;
  double kt0 = 0., kt1 = 0.;
  if (ok && wood) {
    slope_stencil(x1v, n, wt0, wt1, wt2, i0);
    for (int i = 0; i < n; ++i) {
      double h = x1f[i + 1] - x1f[i];
      gv[i] = grav * (h * h / 12.);
    }
    for (int i = 0; i < n; ++i) {
      double bm = i == 0 ? wt0[0] : (i == n - 1 ? wt2[n - 1] : wt1[i]);
      double bl = i == 0 ? 0. : (i == n - 1 ? wt1[n - 1] : wt0[i]);
      double bh = i == n - 1 ? 0. : (i == 0 ? wt1[0] : wt2[i]);
      kmid[i] = gv[i] * bm;
      klo[i] = i >= 1 ? bl * gv[i] : 0.;
      khi[i] = i <= n - 2 ? bh * gv[i] : 0.;
    }
    kt0 = gv[0] * wt2[0];
    kt1 = gv[n - 1] * wt0[n - 1];
    for (int i = 0; i < n; ++i) {
      if (partial) {
        A3[i][2][0] -= kmid[i] / dtc;
        B3[i][2][0] -= klo[i] / dtc;
        C3[i][2][0] -= khi[i] / dtc;
        continue;
      }
      A[i][4][0] -= kmid[i] / dtc;
      B[i][4][0] -= klo[i] / dtc;
      C[i][4][0] -= khi[i] / dtc;
    }
    /* du[IPR] -= K du0[IDN] (GravityWork::apply_rows) */
    double* s = malloc(sizeof(double) * n);
    for (int i = 0; i < n; ++i) s[i] = kmid[i] * du0[i];
    for (int i = 1; i < n; ++i) s[i] += klo[i] * du0[i - 1];
    for (int i = 0; i < n - 1; ++i) s[i] += khi[i] * du0[i + 1];
    s[0] += kt0 * du0[2];
    s[n - 1] += kt1 * du0[n - 3];
    for (int i = 0; i < n; ++i) DU(4, i) -= s[i];
    free(s);
  }
  /* (3p) the partial matrix's forward sweep (ForwardSweep, N = 3): the
   * right-hand side less the assembly's m_t term, the block inverted
   * explicitly after the LU screen; then back substitution and Woodbury on
   * the 3-vectors.  The solution goes to dl rows 0, 1, 4; the tangential
   * rows keep the explicit du */
  for (int i = 0; i < n && ok && partial; ++i) {
    double rhs[3] = {DU(0, i) / dtc, DU(1, i) / dtc, DU(4, i) / dtc};
    for (int r = 0; r < 3; ++r)
      if (rc[i][r] != 0) rhs[r] -= rc[i][r];
    if (i > 0) {
      M3 t;
      mat3_mul(t, B3[i], A3[i - 1]);
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) A3[i][r][c] -= t[r][c];
    }
    M3 LU, inv;
    memcpy(LU, A3[i], sizeof(M3));
    if (ludcmp3(LU) == 0) {
      ok = 0;
      break;
    }
    inverse3(inv, A3[i]);
    double t[3], u[3];
    if (i > 0) {
      mat3_vec(u, B3[i], d3[i - 1]);
      for (int r = 0; r < 3; ++r) t[r] = rhs[r] - u[r];
    } else {
      for (int r = 0; r < 3; ++r) t[r] = rhs[r];
    }
    mat3_vec(d3[i], inv, t);
    if (wood) {
      double e0[3] = {0, 0, i == 0 ? 1. : 0.}, e1[3] = {0, 0, i == n - 1 ? 1. : 0.};
      if (i > 0) {
        mat3_vec(u, B3[i], y0[i - 1]);
        for (int r = 0; r < 3; ++r) t[r] = e0[r] - u[r];
      } else {
        for (int r = 0; r < 3; ++r) t[r] = e0[r];
      }
      mat3_vec(y0[i], inv, t);
      if (i > 0) {
        mat3_vec(u, B3[i], y1[i - 1]);
        for (int r = 0; r < 3; ++r) t[r] = e1[r] - u[r];
      } else {
        for (int r = 0; r < 3; ++r) t[r] = e1[r];
      }
      mat3_vec(y1[i], inv, t);
    }
    M3 ap;
    mat3_mul(ap, inv, C3[i]);
    memcpy(A3[i], ap, sizeof(M3));
    for (int r = 0; r < 3; ++r) {
      if (!isfinite(d3[i][r])) ok = 0;
      for (int c = 0; c < 3; ++c)
        if (!isfinite(A3[i][r][c])) ok = 0;
    }
  }
  if (ok && partial) {
    /* vic_backward_substitute: each vector only if its first layer is
     * finite */
    int f0 = 1, f1 = 1;
    for (int r = 0; r < 3 && wood; ++r) {
      if (!isfinite(y0[0][r])) f0 = 0;
      if (!isfinite(y1[0][r])) f1 = 0;
    }
    for (int i = n - 2; i >= 0; --i) {
      double t[3];
      mat3_vec(t, A3[i], d3[i + 1]);
      for (int r = 0; r < 3; ++r) d3[i][r] -= t[r];
      if (wood && f0) {
        mat3_vec(t, A3[i], y0[i + 1]);
        for (int r = 0; r < 3; ++r) y0[i][r] -= t[r];
      }
      if (wood && f1) {
        mat3_vec(t, A3[i], y1[i + 1]);
        for (int r = 0; r < 3; ++r) y1[i][r] -= t[r];
      }
    }
    if (wood) {
      double k0 = -kt0 / dtc, k1 = -kt1 / dtc;
      k0 = k0 * 1.;
      k1 = k1 * 1.;
      int a0 = 2, a1 = n - 3;
      double m00 = 1. + k0 * y0[a0][0], m01 = k0 * y1[a0][0];
      double m10 = k1 * y0[a1][0], m11 = 1. + k1 * y1[a1][0];
      double r0 = k0 * d3[a0][0], r1 = k1 * d3[a1][0];
      double det = m00 * m11 - m01 * m10;
      double al0 = (m11 * r0 - m01 * r1) / det, al1 = (m00 * r1 - m10 * r0) / det;
      for (int i = 0; i < n; ++i)
        for (int r = 0; r < 3; ++r) {
          d3[i][r] -= y0[i][r] * al0;
          d3[i][r] -= y1[i][r] * al1;
        }
    }
    for (int i = 0; i < n; ++i) {
      dl[i][0] = d3[i][0];
      dl[i][1] = d3[i][1];
      dl[i][2] = DU(2, i);
      dl[i][3] = DU(3, i);
      dl[i][4] = d3[i][2];
      for (int r = 0; r < 3; ++r)
        if (!isfinite(d3[i][r])) ok = 0;
    }
  }
  /* (3) forward sweep (ForwardSweep<K = 2>, N = 5) */
  for (int i = 0; i < n && ok && !partial; ++i) {
    double rhs[5] = {DU(0, i) / dtc, DU(1, i) / dtc, DU(2, i) / dtc,
                     DU(3, i) / dtc, DU(4, i) / dtc};
    if (i > 0) {
      M5 t;
      mat_mul(t, B[i], A[i - 1]);
      for (int r = 0; r < 5; ++r)
        for (int c = 0; c < 5; ++c) A[i][r][c] -= t[r][c];
    }
    M5 LU;
    memcpy(LU, A[i], sizeof(M5));
    int indx[5] = {0, 1, 2, 3, 4};
    if (ludcmp5(LU, indx) == 0) {
      ok = 0;
      break;
    }
    double sol[5][8];
    int m = wood ? 8 : 6;
    for (int r = 0; r < 5; ++r)
      for (int c = 0; c < 5; ++c) sol[r][c] = C[i][r][c];
    double e0[5] = {0, 0, 0, 0, i == 0 ? 1. : 0.};
    double e1[5] = {0, 0, 0, 0, i == n - 1 ? 1. : 0.};
    if (i > 0) {
      V5 t;
      mat_vec(t, B[i], dl[i - 1]);
      for (int r = 0; r < 5; ++r) sol[r][5] = rhs[r] - t[r];
      if (wood) {
        mat_vec(t, B[i], z0[i - 1]);
        for (int r = 0; r < 5; ++r) sol[r][6] = e0[r] - t[r];
        mat_vec(t, B[i], z1[i - 1]);
        for (int r = 0; r < 5; ++r) sol[r][7] = e1[r] - t[r];
      }
    } else {
      for (int r = 0; r < 5; ++r) {
        sol[r][5] = rhs[r];
        sol[r][6] = e0[r];
        sol[r][7] = e1[r];
      }
    }
    lubksb5(LU, indx, sol, m);
    for (int r = 0; r < 5; ++r)
      for (int c = 0; c < m; ++c)
        if (!isfinite(sol[r][c])) ok = 0;
    if (!ok) break;
    for (int r = 0; r < 5; ++r) {
      for (int c = 0; c < 5; ++c) A[i][r][c] = sol[r][c];
      dl[i][r] = sol[r][5];
      if (wood) {
        z0[i][r] = sol[r][6];
        z1[i][r] = sol[r][7];
      }
    }
  }
  if (ok && !partial) {
    /* (4) back substitution */
    for (int i = n - 2; i >= 0; --i) {
      V5 t;
      mat_vec(t, A[i], dl[i + 1]);
      for (int r = 0; r < 5; ++r) dl[i][r] -= t[r];
      if (wood) {
        mat_vec(t, A[i], z0[i + 1]);
        for (int r = 0; r < 5; ++r) z0[i][r] -= t[r];
        mat_vec(t, A[i], z1[i + 1]);
        for (int r = 0; r < 5; ++r) z1[i][r] -= t[r];
      }
    }
    /* (5) Woodbury: the wall third points of the slope */
    if (wood) {
      double k0 = -kt0 / dtc, k1 = -kt1 / dtc;
      k0 = k0 * 1.;
      k1 = k1 * 1.;
      int a0 = 2, a1 = n - 3;
      double m00 = 1. + k0 * z0[a0][0], m01 = k0 * z1[a0][0];
      double m10 = k1 * z0[a1][0], m11 = 1. + k1 * z1[a1][0];
      double r0 = k0 * dl[a0][0], r1 = k1 * dl[a1][0];
      double det = m00 * m11 - m01 * m10;
      double al0 = (m11 * r0 - m01 * r1) / det, al1 = (m00 * r1 - m10 * r0) / det;
      for (int i = 0; i < n; ++i)
        for (int r = 0; r < 5; ++r) {
          dl[i][r] -= z0[i][r] * al0;
          dl[i][r] -= z1[i][r] * al1;
        }
    }
    for (int i = 0; i < n && ok; ++i)
      for (int r = 0; r < 5; ++r)
        if (!isfinite(dl[i][r])) ok = 0;
  }
  if (ok) {
    /* (6) redistribution: the constituent column (no species), then the
     * per-cell map */
    double* mf_dn = calloc(n, sizeof(double));   /* MASS(IDN) */
    double* mf_M = calloc(n + 1, sizeof(double)); /* MASS(IVX): face below i */
    double* mf_q = calloc(n + 1, sizeof(double)); /* MASS(IVZ): moved total */
    double* vols = malloc(sizeof(double) * n);
    for (int i = 0; i < n; ++i) vols[i] = vol;
    redistribute_column(n, w, st, du, dl, vols, partial, mf_dn, mf_M, mf_q);
    free(vols);
    /* (7) book_remainder_: projection and clamp work, then the corrected-PE
     * remainder g1 sigma^2 s[du - du0] beyond what the matrix booked */
    for (int i = 0; i < n; ++i) {
      double projected = (mf_M[i] - mf_M[i + 1]) / vol;
      double ph = -grav * x1v[i];
      double pw = ph * (dl[i][0] - du0[i] - projected);
      double dp_lo = -grav * (x1f[i] - x1v[i]);
      double dp_hi = -grav * (x1f[i + 1] - x1v[i]);
      double mv_lo = mf_q[i] - mf_M[i], mv_hi = mf_q[i + 1] - mf_M[i + 1];
      double cw = -(dp_hi * mv_hi - dp_lo * mv_lo) / vol;
      DU(4, i) += pw + cw;
    }
    if (wood) {
      double* mv = malloc(sizeof(double) * n);
      double* rw = malloc(sizeof(double) * n);
      for (int i = 0; i < n; ++i) mv[i] = DU(0, i) - du0[i];
      for (int i = 0; i < n; ++i) rw[i] = dl[i][0] - du0[i];
      for (int i = 0; i < n; ++i) {
        double sl = wt0[i] * mv[i0[i]];
        sl += wt1[i] * mv[i0[i] + 1];
        sl += wt2[i] * mv[i0[i] + 2];
        double work = gv[i] * sl;
        double s = kmid[i] * rw[i];
        if (i >= 1) s += klo[i] * rw[i - 1];
        if (i <= n - 2) s += khi[i] * rw[i + 1];
        if (i == 0) s += kt0 * rw[2];
        if (i == n - 1) s += kt1 * rw[n - 3];
        work -= s;
        DU(4, i) += work;
      }
      free(mv);
      free(rw);
    }
    if (t1) {
      /* "vic.mass_dry": the clamped dry transfer q of each face over dt A
       * (zero on the walls), row IDN; "vic.momentum_t" (full matrix): minus
       * the prefix of V (du - du0) of the tangential rows from the bottom
       * wall, top face included, over dt A, rows IVY and IVZ */
      for (int f = 0; f <= n; ++f)
        t1[OG_IDN * st + f] = t1[OG_IDN * st + f] + mf_q[f] / kdt;
      /* partial matrix: "vic.momentum_t" is the donor transfer q w_t */
      for (int f = 0; f <= n && partial; ++f) {
        double q = mf_q[f];
        int donor = q > 0. ? f - 1 : f;
        t1[OG_IVY * st + f] = t1[OG_IVY * st + f] + q * WV(2, donor) / kdt;
        t1[OG_IVZ * st + f] = t1[OG_IVZ * st + f] + q * WV(3, donor) / kdt;
      }
      double sy = 0., sz = 0.;
      for (int f = 0; f <= n && !partial; ++f) {
        double py = 0., pz = 0.;
        if (f > 0) {
          sy = sy + (dl[f - 1][2] - du0[2 * n + f - 1]) * vol;
          sz = sz + (dl[f - 1][3] - du0[3 * n + f - 1]) * vol;
          py = -sy;
          pz = -sz;
        }
        t1[OG_IVY * st + f] = t1[OG_IVY * st + f] + py / kdt;
        t1[OG_IVZ * st + f] = t1[OG_IVZ * st + f] + pz / kdt;
      }
    }
    if (qout)
      for (int f = 0; f <= n; ++f) qout[f] = mf_q[f];
    free(mf_dn);
    free(mf_M);
    free(mf_q);
  }
  if (!ok) /* a failed column keeps the explicit tendency */
    for (int v = 0; v < 5; ++v)
      for (int i = 0; i < n; ++i) DU(v, i) = du0[v * n + i];
#undef WV
#undef DU
  free(A); free(B); free(C); free(dl); free(z0); free(z1); free(du0);
  free(kmid); free(klo); free(khi); free(gv); free(wt0); free(wt1); free(wt2);
  free(i0);
  free(A3); free(B3); free(C3); free(rc); free(d3); free(y0); free(y1);
  return ok ? 0 : 1;
}

int og_implicit(const og_block* b, const double* w, double dtc, double* du) {
  return og_implicit_reg(b, w, dtc, du, NULL, 0.);
}

int og_implicit_reg(const og_block* b, const double* w, double dtc, double* du,
                    double* t1, double dt) {
  const int n1 = b->nc1, n2 = b->nc2, ng = b->ng;
  const size_t nc = (size_t)n1 * n2 * b->nc3;
  const int jl = n2 > 1 ? ng : 0, ju1 = n2 > 1 ? n2 - ng : 1;
  const int n3 = b->nc3, kl = n3 > 1 ? ng : 0, ku1 = n3 > 1 ? n3 - ng : 1;
  const int n = n1 - 2 * ng;
  const long nj = ju1 - jl, ncols = nj * (ku1 - kl);
  int failed = 0;
  /* every (x2, x3) column of the interior */
#pragma omp parallel for schedule(static) reduction(+ : failed)
  for (long cidx = 0; cidx < ncols; ++cidx) {
    int j = jl + (int)(cidx % nj), k = kl + (int)(cidx / nj);
    size_t c = ((size_t)k * n2 + j) * n1 + ng;
    failed += vic_column(b, w + c, nc, du + c, n, dtc, b->x1f + ng, b->x1v + ng,
                         t1 ? t1 + c : NULL, dt * (b->dx3 * b->dx2),
                         b->vic_q ? b->vic_q + c : NULL);
  }
  return failed;
}
