// The vertical implicit correction (VIC) of the hydro stage, FP64, the full
// 5x5 block-tridiagonal scheme (integration/implicit-scheme 9) on Cartesian
// blocks without solids or species.  Included by sg_stage.cu inside its
// anonymous namespace, once per storage type `real`; the solve always
// computes in FP64.
//
// Reference (paths inside the snapy project):
//   src/implicit/implicit_hydro.cpp:301-560   forward_masked
//   src/implicit/vic_assemble_impl.h:45-214   the blocks a, b, c of a cell
//   src/implicit/flux_decomposition_impl.h    Roe average, |A|, Jacobians
//   src/implicit/vic_gravity_work_impl.h      the energy row's face work
//   src/hydro/gravity_work.hpp:300-366        the corrected-PE rows K
//   src/implicit/forward_sweep_impl.h:30-131  block-Thomas forward sweep
//   src/math/ludcmp.h, src/math/lubksb.h      scaled partial-pivot LU
//   src/implicit/vic_kernels.h:100-160        back substitution, Woodbury
//   src/implicit/vic_redistribute_impl.h      constituent column, cell map
//   src/implicit/implicit_hydro.cpp:713-792   the gravity-work remainder
// Three launches per stage, as the work's parallelism dictates: the blocks
// of every cell in parallel (vic_assemble_kernel, one thread per cell), the
// serial block-Thomas sweep of each column (vic_solve_kernel, one WARP per
// column: the 5x5 block products run one entry per lane through warp
// shuffles, the 8 right-hand sides of the LU back-solve one per lane, the
// factorisation on the warp's shared-memory tile), and the column's
// redistribution, remainder and RK combine (vic_finish_kernel, one warp per
// column).  Every product is summed in index order, so the results are bit
// for bit the CPU oracle's.
#pragma once

struct VicScratch {
  double *du, *du0, *A, *B, *C, *D, *Z0, *Z1;
  size_t cells;
};

__device__ __forceinline__ VicScratch vic_scratch(const BlockDev& B) {
  VicScratch s;
  const int ng = B.ng;
  const size_t nx1 = B.nc1 - 2 * ng;
  const size_t nx2 = B.nc2 > 1 ? B.nc2 - 2 * ng : 1;
  s.cells = nx1 * nx2;
  s.du = B.vic;
  s.du0 = s.du + 5 * s.cells;
  s.A = s.du0 + 5 * s.cells;
  s.B = s.A + 25 * s.cells;
  s.C = s.B + 25 * s.cells;
  s.D = s.C + 25 * s.cells;
  s.Z0 = s.D + 5 * s.cells;
  s.Z1 = s.Z0 + 5 * s.cells;
  return s;
}

// bit of the per-block status word: a column's solve failed this step
constexpr int kVicFailed = 32;

__device__ __forceinline__ void vmat_mul(const double* a, const double* b,
                                         double* out) {
#pragma unroll
  for (int r = 0; r < 5; ++r)
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      double s = a[r * 5] * b[c];
#pragma unroll
      for (int k = 1; k < 5; ++k) s += a[r * 5 + k] * b[k * 5 + c];
      out[r * 5 + c] = s;
    }
}

__device__ __forceinline__ void vflux_jacobian(double* J, double gm1,
                                               const double* w) {
  double v1 = w[1], v2 = w[2], v3 = w[3], rho = w[0], pres = w[4];
  double s2 = v1 * v1 + v2 * v2 + v3 * v3;
  double c1 = ((gm1 - 1) * s2 / 2 - (gm1 + 1) / gm1 * pres / rho) * v1;
  double c2 = (gm1 + 1) / gm1 * pres / rho + s2 / 2 - gm1 * v1 * v1;
  J[0] = 0; J[1] = 1.; J[2] = 0.; J[3] = 0.; J[4] = 0.;
  J[5] = gm1 * s2 / 2 - v1 * v1; J[6] = (2. - gm1) * v1; J[7] = -gm1 * v2;
  J[8] = -gm1 * v3; J[9] = gm1;
  J[10] = -v1 * v2; J[11] = v2; J[12] = v1; J[13] = 0.; J[14] = 0.;
  J[15] = -v1 * v3; J[16] = v3; J[17] = 0.; J[18] = v1; J[19] = 0.;
  J[20] = c1; J[21] = c2; J[22] = -gm1 * v2 * v1; J[23] = -gm1 * v3 * v1;
  J[24] = (gm1 + 1) * v1;
}

// |A| = R |Lambda| R^-1 at the face between wl and wr (Roe average)
__device__ __forceinline__ void vabs_jacobian(double* A, double gm1,
                                              const double* wl,
                                              const double* wr) {
  double sqrtdl = sqrt(wl[0]), sqrtdr = sqrt(wr[0]);
  double isdlpdr = 1.0 / (sqrtdl + sqrtdr);
  double pr[5];
  pr[0] = sqrtdl * sqrtdr;
  pr[1] = (sqrtdl * wl[1] + sqrtdr * wr[1]) * isdlpdr;
  pr[2] = (sqrtdl * wl[2] + sqrtdr * wr[2]) * isdlpdr;
  pr[3] = (sqrtdl * wl[3] + sqrtdr * wr[3]) * isdlpdr;
  double el = wl[4] / gm1 +
              0.5 * wl[0] * (wl[1] * wl[1] + wl[2] * wl[2] + wl[3] * wl[3]);
  double er = wr[4] / gm1 +
              0.5 * wr[0] * (wr[1] * wr[1] + wr[2] * wr[2] + wr[3] * wr[3]);
  double hbar = ((el + wl[4]) / sqrtdl + (er + wr[4]) / sqrtdr) * isdlpdr;
  pr[4] = (hbar - 0.5 * (pr[1] * pr[1] + pr[2] * pr[2] + pr[3] * pr[3])) *
          gm1 / (gm1 + 1.) * pr[0];
  double cs = sqrt(pr[4] * (gm1 + 1.) / pr[0]);
  double r = pr[0], u = pr[1], v = pr[2], w = pr[3], p = pr[4];
  double lam[5] = {fabs(u - cs), fabs(u), fabs(u + cs), fabs(u), fabs(u)};
  double ke = 0.5 * (u * u + v * v + w * w);
  double hp = (gm1 + 1.) / gm1 * p / r;
  double h = hp + ke;
  const double R[25] = {1.,         1., 1.,         0., 0.,  //
                        u - cs,     u,  u + cs,     0., 0.,  //
                        v,          v,  v,          1., 0.,  //
                        w,          w,  w,          0., 1.,  //
                        h - u * cs, ke, h + u * cs, v,  w};
  const double Ri[25] = {(cs * ke + u * hp) / (2. * cs * hp),
                         (-hp - cs * u) / (2. * cs * hp),
                         -v / (2. * hp),
                         -w / (2. * hp),
                         1. / (2. * hp),
                         (hp - ke) / hp,
                         u / hp,
                         v / hp,
                         w / hp,
                         -1. / hp,
                         (cs * ke - u * hp) / (2. * cs * hp),
                         (hp - cs * u) / (2. * cs * hp),
                         -v / (2. * hp),
                         -w / (2. * hp),
                         1. / (2. * hp),
                         -v, 0., 1., 0., 0.,
                         -w, 0., 0., 1., 0.};
  double RL[25];
#pragma unroll
  for (int i = 0; i < 5; ++i)
#pragma unroll
    for (int k = 0; k < 5; ++k) RL[i * 5 + k] = R[i * 5 + k] * lam[k];
  vmat_mul(RL, Ri, A);
}

// the primitives of layer i of a column (u of the storage type -> FP64 W)
__device__ __forceinline__ void vic_prim(const real* u, size_t plane,
                                         size_t cell, double gammad,
                                         double* w) {
  double uc[NHYDRO];
#pragma unroll
  for (int v = 0; v < NHYDRO; ++v) uc[v] = (double)u[v * plane + cell];
  cons2prim<double>(uc, w, gammad);
}

// the corrected-PE slope weights of layer k of n (centres x)
__device__ __forceinline__ void vic_slope(const double* x, int n, int k,
                                          double* wt, int* i0) {
  if (k == 0) {
    double a = x[1] - x[0], b = x[2] - x[1];
    wt[0] = -(2. * a + b) / (a * (a + b));
    wt[1] = (a + b) / (a * b);
    wt[2] = -(a / ((a + b) * b));
  } else if (k == n - 1) {
    double c = x[n - 2] - x[n - 3], d = x[n - 1] - x[n - 2];
    wt[0] = d / (c * (c + d));
    wt[1] = -((c + d) / (c * d));
    wt[2] = (c + 2. * d) / ((c + d) * d);
  } else {
    double hm = x[k] - x[k - 1], hp = x[k + 1] - x[k];
    wt[0] = -hp / (hm * (hm + hp));
    wt[1] = (hp - hm) / (hm * hp);
    wt[2] = hm / (hp * (hm + hp));
  }
  int kc = k < 1 ? 1 : (k > n - 2 ? n - 2 : k);
  *i0 = kc - 1;
}

// the K rows of layer k: mid, lo, hi bands and the wall third points
struct VicK {
  double mid, lo, hi, t0, t1, gv;
};

__device__ __forceinline__ VicK vic_krows(const BlockDev& B, int n, int k) {
  const double* x = B.x1v + B.ng;
  const double* f = B.x1f + B.ng;
  VicK K;
  double wt[3];
  int i0;
  vic_slope(x, n, k, wt, &i0);
  double h = f[k + 1] - f[k];
  double gv = B.grav1 * (h * h / 12.);
  double bm = k == 0 ? wt[0] : (k == n - 1 ? wt[2] : wt[1]);
  double bl = k == 0 ? 0. : (k == n - 1 ? wt[1] : wt[0]);
  double bh = k == n - 1 ? 0. : (k == 0 ? wt[1] : wt[2]);
  K.gv = gv;
  K.mid = gv * bm;
  K.lo = k >= 1 ? bl * gv : 0.;
  K.hi = k <= n - 2 ? bh * gv : 0.;
  K.t0 = K.t1 = 0.;
  if (k == 0) K.t0 = gv * wt[2];
  if (k == n - 1) K.t1 = gv * wt[0];
  return K;
}

// (1) the blocks of every interior cell, the K coupling in their (IPR, IDN)
// entries and du[IPR] -= K du0[IDN]
__global__ void __launch_bounds__(kThreads)
    vic_assemble_kernel(const BlockDev* __restrict__ tab, StageParams p) {
  const BlockDev& B = tab[blockIdx.y];
  if (!B.implicit) return;
  const VicScratch S = vic_scratch(B);
  const int ng = B.ng, nc1 = B.nc1, n = nc1 - 2 * ng;
  const size_t plane = (size_t)nc1 * B.nc2 * B.nc3;
  const real* uin = static_cast<const real*>(B.buf[p.in]);
  const double dtc = p.w2 * p.dt[blockIdx.y];
  const double grav = B.grav1, gm1 = B.gammad - 1.;
  const double area = B.dx3 * B.dx2, vol = B.dx3 * (B.dx2 * B.dx1);
  const double* x1v = B.x1v + ng;
  const double* x1f = B.x1f + ng;
  const bool wood = n >= 3;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < S.cells;
       e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % n);
    const size_t col = e / n;
    const size_t jrow = B.nc2 > 1 ? col + ng : 0;
    const size_t base = jrow * nc1 + ng;  // padded cell of layer 0
    double wl[5], wr[5], wn[5];
    vic_prim(uin, plane, base + i - 1, B.gammad, wl);
    vic_prim(uin, plane, base + i, B.gammad, wr);
    vic_prim(uin, plane, base + i + 1, B.gammad, wn);
    double Jp[25], Jc[25], Jn[25], Am[25], Ap[25];
    vflux_jacobian(Jp, gm1, wl);
    vflux_jacobian(Jc, gm1, wr);
    vabs_jacobian(Am, 0.5 * (B.gammad + B.gammad) - 1., wl, wr);
    vflux_jacobian(Jn, gm1, wn);
    vabs_jacobian(Ap, 0.5 * (B.gammad + B.gammad) - 1., wr, wn);
    const double half_inv_vol = 0.5 / vol;
    const double lower = 0.5 * area * (x1v[i] - x1f[i]) / vol;
    const double upper = 0.5 * area * (x1f[i + 1] - x1v[i]) / vol;
    double a[25], b[25], c[25];
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
      for (int q = 0; q < 5; ++q) {
        const int k = r * 5 + q;
        double phi = (r == 1 && q == 0) || (r == 4 && q == 1) ? grav : 0.;
        a[k] = (Am[k] * area + Ap[k] * area + (area - area) * Jc[k]) *
                   half_inv_vol - phi;
        b[k] = -(Am[k] + Jp[k]) * area * half_inv_vol;
        c[k] = -(Ap[k] - Jn[k]) * area * half_inv_vol;
      }
    const double rdt = 1. / dtc;
#pragma unroll
    for (int r = 0; r < 5; ++r) a[r * 5 + r] += rdt;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      a[20 + k] -= grav * (upper * Ap[k] - lower * Am[k]);
      b[20 + k] -= grav * lower * Am[k];
      c[20 + k] += grav * upper * Ap[k];
    }
    a[21] += grav * (1. - lower - upper);
    b[21] -= grav * lower;
    c[21] -= grav * upper;
    const double bnd[5] = {1., -1., 1., 1., 1.};
    if (i == 0)
#pragma unroll
      for (int r = 0; r < 5; ++r)
#pragma unroll
        for (int q = 0; q < 5; ++q) a[r * 5 + q] += b[r * 5 + q] * bnd[q];
    if (i == n - 1)
#pragma unroll
      for (int r = 0; r < 5; ++r)
#pragma unroll
        for (int q = 0; q < 5; ++q) a[r * 5 + q] += c[r * 5 + q] * bnd[q];
    const size_t cell = col * n + i;
    double du0[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      du0[v] = S.du[v * S.cells + cell];
      S.du0[v * S.cells + cell] = du0[v];
    }
    if (wood) {
      VicK K = vic_krows(B, n, i);
      a[20] -= K.mid / dtc;
      b[20] -= K.lo / dtc;
      c[20] -= K.hi / dtc;
      // du[IPR] -= (K du0[IDN])_i : the IDN row is read only
      const double* dn = S.du + col * n;
      double s = K.mid * dn[i];
      if (i >= 1) s += K.lo * dn[i - 1];
      if (i <= n - 2) s += K.hi * dn[i + 1];
      if (i == 0) s += K.t0 * dn[2];
      if (i == n - 1) s += K.t1 * dn[n - 3];
      S.du[4 * S.cells + cell] = du0[4] - s;
    }
#pragma unroll
    for (int k = 0; k < 25; ++k) {
      S.A[cell * 25 + k] = a[k];
      S.B[cell * 25 + k] = b[k];
      S.C[cell * 25 + k] = c[k];
    }
  }
}

// ludcmp<double, 5, Implicit> on a row-major 5x5 in shared memory
// (src/math/ludcmp.h); one lane runs it
__device__ __forceinline__ int vludcmp(double* a, int* indx) {
  int i, imax = 0, j, k, d;
  double big, dum, sum, temp, vv[5], scale[5];
  const double tolerance = 8. * 5 * 2.220446049250313e-16;
  for (int q = 0; q < 25; ++q)
    if (!isfinite(a[q])) return 0;
  d = 1;
  for (i = 0; i < 5; i++) {
    big = 0.0;
    for (j = 0; j < 5; j++)
      if ((temp = fabs(a[i * 5 + j])) > big) big = temp;
    if (big == 0.0) return 0;
    scale[i] = big;
    vv[i] = 1.0 / big;
    if (!isfinite(vv[i])) return 0;
  }
  for (j = 0; j < 5; j++) {
    for (i = 0; i < j; i++) {
      sum = a[i * 5 + j];
      for (k = 0; k < i; k++) sum -= a[i * 5 + k] * a[k * 5 + j];
      if (!isfinite(sum)) return 0;
      a[i * 5 + j] = sum;
    }
    big = 0.0;
    for (i = j; i < 5; i++) {
      sum = a[i * 5 + j];
      for (k = 0; k < j; k++) sum -= a[i * 5 + k] * a[k * 5 + j];
      if (!isfinite(sum)) return 0;
      a[i * 5 + j] = sum;
      dum = vv[i] * fabs(sum);
      if (!isfinite(dum)) return 0;
      if (dum >= big) {
        big = dum;
        imax = i;
      }
    }
    if (j != imax) {
      for (k = 0; k < 5; k++) {
        dum = a[imax * 5 + k];
        a[imax * 5 + k] = a[j * 5 + k];
        a[j * 5 + k] = dum;
      }
      d = -d;
      vv[imax] = vv[j];
      temp = scale[imax];
      scale[imax] = scale[j];
      scale[j] = temp;
    }
    indx[j] = imax;
    if (fabs(a[j * 5 + j]) / scale[j] <= tolerance) return 0;
    if (j != 4) {
      dum = (1.0 / a[j * 5 + j]);
      for (i = j + 1; i < 5; i++) a[i * 5 + j] *= dum;
    }
  }
  for (int q = 0; q < 25; ++q)
    if (!isfinite(a[q])) return 0;
  return d;
}

constexpr int kVicWarps = 4;  // columns per CTA of the solve and finish

// the per-warp shared tile of the sweep
struct VicWarpTile {
  double lu[25];      // a[i] - b[i] a'[i-1], factorised in place
  double bm[25];      // b[i]
  double sol[5 * 8];  // [row][col]: c[i] | rhs - b d' | e0 - b z0 | e1 - b z1
  double prev[3 * 5];  // d, z0, z1 of layer i - 1
  int indx[5];
  int ok;
};

// (2) the block-Thomas sweep, back substitution and Woodbury update of
// each column, one warp per column
__global__ void __launch_bounds__(32 * kVicWarps)
    vic_solve_kernel(const BlockDev* __restrict__ tab, StageParams p,
                     int* status) {
  __shared__ VicWarpTile tiles[kVicWarps];
  const BlockDev& B = tab[blockIdx.y];
  if (!B.implicit) return;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  VicWarpTile& T = tiles[wid];
  const VicScratch S = vic_scratch(B);
  const int ng = B.ng, n = B.nc1 - 2 * ng;
  const size_t ncol = S.cells / n;
  const size_t col = (size_t)blockIdx.x * kVicWarps + wid;
  if (col >= ncol) return;  // whole warps leave together
  const double dtc = p.w2 * p.dt[blockIdx.y];
  const bool wood = n >= 3;
  const int m = wood ? 8 : 6;
  double* A = S.A + col * n * 25;
  const double* Bm = S.B + col * n * 25;
  const double* C = S.C + col * n * 25;
  double* D = S.D + col * n * 5;
  double* Z0 = S.Z0 + col * n * 5;
  double* Z1 = S.Z1 + col * n * 5;
  const int r = lane / 5, c = lane % 5;  // lane < 25 owns entry (r, c)
  // the input screen: du of every layer finite
  bool fin = true;
  for (int e = lane; e < 5 * n; e += 32)
    fin = fin && isfinite(S.du[(e / n) * S.cells + col * n + (e % n)]);
  bool ok = __all_sync(0xffffffffu, fin);
  double aprev = 0.;  // a'[i-1] entry (r, c) of this lane
  for (int i = 0; i < n && ok; ++i) {
    const size_t cell = col * n + i;
    double aij = 0., bij = 0.;
    if (lane < 25) {
      aij = A[i * 25 + lane];
      bij = Bm[i * 25 + lane];
      T.bm[lane] = bij;
      T.sol[r * 8 + c] = C[i * 25 + lane];
    }
    // a[i] -= b[i] a'[i-1], entry (r, c) summed over k in order
    if (i > 0) {
      double t = 0.;
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        double bk = __shfl_sync(0xffffffffu, bij, r * 5 + k);
        double ak = __shfl_sync(0xffffffffu, aprev, k * 5 + c);
        t = k == 0 ? bk * ak : t + bk * ak;
      }
      aij -= t;
    }
    if (lane < 25) T.lu[lane] = aij;
    __syncwarp();
    // the right-hand sides: lane q5 * 5 + rr (q5 < 3) forms column 5 + q5
    if (lane < 15) {
      const int q5 = lane / 5, rr = lane % 5;
      double base;
      if (q5 == 0)
        base = S.du[rr * S.cells + cell] / dtc;
      else
        base = (rr == 4 && ((q5 == 1 && i == 0) || (q5 == 2 && i == n - 1)))
                   ? 1. : 0.;
      if (i > 0) {
        const double* v = T.prev + q5 * 5;
        double t = T.bm[rr * 5] * v[0];
#pragma unroll
        for (int k = 1; k < 5; ++k) t += T.bm[rr * 5 + k] * v[k];
        base = base - t;
      }
      T.sol[rr * 8 + 5 + q5] = base;
    }
    __syncwarp();
    if (lane == 0) {
#pragma unroll
      for (int q = 0; q < 5; ++q) T.indx[q] = q;
      T.ok = vludcmp(T.lu, T.indx) != 0;
    }
    __syncwarp();
    if (!T.ok) {
      ok = false;
      break;
    }
    // lubksb on the m right-hand sides, one column per lane
    if (lane < m) {
      const int q = lane;
      double* s = T.sol;
      for (int rr = 0; rr < 5; ++rr) {
        int ip = T.indx[rr];
        if (ip != rr) {
          double tt = s[ip * 8 + q];
          s[ip * 8 + q] = s[rr * 8 + q];
          s[rr * 8 + q] = tt;
        }
        for (int jj = 0; jj < rr; ++jj) s[rr * 8 + q] -= T.lu[rr * 5 + jj] * s[jj * 8 + q];
      }
      for (int rr = 4; rr >= 0; --rr) {
        for (int jj = rr + 1; jj < 5; ++jj)
          s[rr * 8 + q] -= T.lu[rr * 5 + jj] * s[jj * 8 + q];
        s[rr * 8 + q] /= T.lu[rr * 5 + rr];
      }
    }
    __syncwarp();
    bool f = true;
    for (int e = lane; e < 5 * m; e += 32) f = f && isfinite(T.sol[(e / m) * 8 + (e % m)]);
    ok = __all_sync(0xffffffffu, f);
    if (!ok) break;
    if (lane < 25) {
      aprev = T.sol[r * 8 + c];
      A[i * 25 + lane] = aprev;
    }
    if (lane < 15) {
      const int q5 = lane / 5, rr = lane % 5;
      double v = T.sol[rr * 8 + 5 + q5];
      (q5 == 0 ? D : (q5 == 1 ? Z0 : Z1))[i * 5 + rr] = v;
      T.prev[q5 * 5 + rr] = v;
    }
    __syncwarp();
  }
  if (ok) {
    // back substitution: d[i] -= a'[i] d[i+1] (and z0, z1); lane q5*5+rr
    // owns row rr of vector q5, the running vector in T.prev
    for (int i = n - 2; i >= 0; --i) {
      if (lane < 25) T.lu[lane] = A[i * 25 + lane];
      __syncwarp();
      double v = 0.;
      if (lane < 15) {
        const int q5 = lane / 5, rr = lane % 5;
        const double* x = T.prev + q5 * 5;
        double t = T.lu[rr * 5] * x[0];
#pragma unroll
        for (int k = 1; k < 5; ++k) t += T.lu[rr * 5 + k] * x[k];
        double* vec = q5 == 0 ? D : (q5 == 1 ? Z0 : Z1);
        v = vec[i * 5 + rr] - t;
        vec[i * 5 + rr] = v;
      }
      __syncwarp();
      if (lane < 15) T.prev[lane] = v;
      __syncwarp();
    }
    if (wood) {
      __syncwarp();
      VicK K0 = vic_krows(B, n, 0), K1 = vic_krows(B, n, n - 1);
      double k0 = -K0.t0 / dtc, k1 = -K1.t1 / dtc;
      k0 = k0 * 1.;
      k1 = k1 * 1.;
      const int a0 = 2, a1 = n - 3;
      double m00 = 1. + k0 * Z0[a0 * 5], m01 = k0 * Z1[a0 * 5];
      double m10 = k1 * Z0[a1 * 5], m11 = 1. + k1 * Z1[a1 * 5];
      double r0 = k0 * D[a0 * 5], r1 = k1 * D[a1 * 5];
      double det = m00 * m11 - m01 * m10;
      double al0 = (m11 * r0 - m01 * r1) / det;
      double al1 = (m00 * r1 - m10 * r0) / det;
      __syncwarp();
      for (int e = lane; e < 5 * n; e += 32) {
        double d = D[e];
        d -= Z0[e] * al0;
        d -= Z1[e] * al1;
        D[e] = d;
      }
    }
    __syncwarp();
    bool f = true;
    for (int e = lane; e < 5 * n; e += 32) f = f && isfinite(D[e]);
    ok = __all_sync(0xffffffffu, f);
  }
  // a failed column is marked in its solution: the finish keeps du0
  if (!ok && lane == 0) {
    D[0] = __longlong_as_double(0x7ff8000000000000ll);
    atomicOr(&status[blockIdx.y], kVicFailed);
  }
}

// (3) redistribution, the gravity-work remainder and the RK combine of each
// column, one warp per column: the serial passes of the constituent column
// (sums, face-mass prefix, availability clamp) on lane 0, the per-layer maps
// on every lane
__global__ void __launch_bounds__(32 * kVicWarps)
    vic_finish_kernel(const BlockDev* __restrict__ tab, StageParams p) {
  const BlockDev& B = tab[blockIdx.y];
  if (!B.implicit) return;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const VicScratch S = vic_scratch(B);
  const int ng = B.ng, nc1 = B.nc1, n = nc1 - 2 * ng;
  const size_t ncol = S.cells / n;
  const size_t col = (size_t)blockIdx.x * kVicWarps + wid;
  if (col >= ncol) return;
  const size_t plane = (size_t)nc1 * B.nc2 * B.nc3;
  const real* uin = static_cast<const real*>(B.buf[p.in]);
  const real* u0 = static_cast<const real*>(B.buf[p.u0]);
  real* uout = static_cast<real*>(B.buf[p.out]);
  const size_t jrow = B.nc2 > 1 ? col + ng : 0;
  const size_t base = jrow * nc1 + ng;
  const double grav = B.grav1;
  const double vol = B.dx3 * (B.dx2 * B.dx1);
  const double* x1v = B.x1v + ng;
  const double* x1f = B.x1f + ng;
  const double* D = S.D + col * n * 5;
  double* du = S.du + col * n;      // row v at du[v * cells + i]
  const double* du0 = S.du0 + col * n;
  const size_t cs = S.cells;
  const bool ok = isfinite(D[0]);
  const bool wood = n >= 3;
  // work arrays of the column, in the (now free) Woodbury scratch
  double* mM = S.Z0 + col * n * 5;  // n + 1: the face mass below layer i
  double* mq = mM + (n + 1);        // n + 1: the moved total mass
  double* mdn = mq + (n + 1);       // n: the dry-gas increment
  double* rho = mdn + n;            // n: the density of each layer
  if (ok) {
    for (int i = lane; i < n; i += 32) {
      double w[5];
      vic_prim(uin, plane, base + i, B.gammad, w);
      rho[i] = w[0];
      mdn[i] = 0.;
      mq[i] = (D[i * 5] - du[i]) * vol;  // staged: phi of layer i
    }
    __syncwarp();
    if (lane == 0) {
      double R = 0, Ssum = 0;
      for (int i = 0; i < n; ++i) {
        R += mq[i];
        Ssum += rho[i] * vol;
      }
      double M = 0;
      for (int i = 0; i < n; ++i) {
        mM[i] = M;
        M -= mq[i] - R * (rho[i] * vol / Ssum);
      }
      mM[n] = 0.;
      for (int i = 0; i <= n; ++i) mq[i] = 0.;
      double avail = (rho[0] * 1. + du[0]) * vol;
      if (avail < 0) avail = 0;
      for (int i = 0; i + 1 < n; ++i) {
        double avail_up = (rho[i + 1] * 1. + du[i + 1]) * vol;
        if (avail_up < 0) avail_up = 0;
        double Mf = mM[i + 1];
        double q = Mf > 0 ? Mf * 1. : Mf * 1.;
        if (q > avail) q = avail;
        if (q < -avail_up) q = -avail_up;
        mdn[i] -= q / vol;
        mdn[i + 1] += q / vol;
        mq[i + 1] = q;
        avail = avail_up + q;
      }
    }
    __syncwarp();
    for (int i = lane; i < n; i += 32) {
      du[i] += mdn[i];
      du[cs + i] = D[i * 5 + 1];
      du[2 * cs + i] = D[i * 5 + 2];
      du[3 * cs + i] = D[i * 5 + 3];
      double e = D[i * 5 + 4];
      double projected = (mM[i] - mM[i + 1]) / vol;
      double ph = -grav * x1v[i];
      double pw = ph * (D[i * 5] - du0[i] - projected);
      double dp_lo = -grav * (x1f[i] - x1v[i]);
      double dp_hi = -grav * (x1f[i + 1] - x1v[i]);
      double mv_lo = mq[i] - mM[i], mv_hi = mq[i + 1] - mM[i + 1];
      double cw = -(dp_hi * mv_hi - dp_lo * mv_lo) / vol;
      du[4 * cs + i] = e + (pw + cw);
    }
    __syncwarp();
    if (wood) {
      // the remainder g1 sigma^2 s[du - du0] - K (raw - du0) of each layer,
      // from the final IDN row of its neighbours
      // staged in mdn (free again): every layer's work reads the IDN row
      // only, so the IPR row is written after all of them
      for (int i = lane; i < n; i += 32) {
        double wt[3];
        int i0;
        vic_slope(x1v, n, i, wt, &i0);
        VicK K = vic_krows(B, n, i);
        double mv0 = du[i0] - du0[i0], mv1 = du[i0 + 1] - du0[i0 + 1],
               mv2 = du[i0 + 2] - du0[i0 + 2];
        double sl = wt[0] * mv0;
        sl += wt[1] * mv1;
        sl += wt[2] * mv2;
        double wk = K.gv * sl;
        auto rw = [&](int k) { return D[k * 5] - du0[k]; };
        double s = K.mid * rw(i);
        if (i >= 1) s += K.lo * rw(i - 1);
        if (i <= n - 2) s += K.hi * rw(i + 1);
        if (i == 0) s += K.t0 * rw(2);
        if (i == n - 1) s += K.t1 * rw(n - 3);
        wk -= s;
        mdn[i] = wk;
      }
      __syncwarp();
      for (int i = lane; i < n; i += 32) du[4 * cs + i] += mdn[i];
    }
    __syncwarp();
  }
  // the RK combine of the column (a failed column keeps the explicit du)
  const double* dsel = ok ? S.du + col * n : du0;
  const real w0 = real(p.w0), w1 = real(p.w1), w2 = real(p.w2);
  for (int i = lane; i < n; i += 32) {
    const size_t c = base + i;
#pragma unroll
    for (int v = 0; v < NHYDRO; ++v) {
      const size_t q = v * plane + c;
      uout[q] = w0 * u0[q] + w1 * uin[q] + w2 * real(dsel[v * cs + i]);
    }
  }
}
