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
// column, or one thread per column when the batch has columns enough to
// fill every SM sub-partition).  Every product is summed in index order, so the results are bit
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
  const size_t nx3 = B.nc3 > 1 ? B.nc3 - 2 * ng : 1;
  s.cells = nx1 * nx2 * nx3;
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

// the refined-solve part of an implicit-precision float32 block's scratch
// (after the FP64 part, 16-byte aligned): per cell the blocks A, B, C in
// FP32 (25 each in rows of 5, padded to 28 for 16-byte loads), the pivot
// blocks' LU factors (25, then the reciprocals of the diagonal (5) and the
// pivot rows packed 3 bits each, padded to 32), the C' blocks (28) and the
// residuals, then the sweep's y, of the three right-hand sides (15 and a
// pad, row v of right-hand side k at 5 k + v); per column the largest update of each
// right-hand side in the last pass (3), the largest |x| of each after the
// first pass (3) and the direct-solve mask
constexpr int kBlk32 = 28;  // floats per cell of A, B, C
constexpr int kLu32 = 32;   // floats per cell of the factors
constexpr int kR32 = 16;    // floats per cell of the residuals (15 and a pad)
struct VicScratch32 {
  float *A, *B, *C, *LU, *CP, *R, *stat;
  int* mask;
  size_t ncol;
};

__device__ __forceinline__ VicScratch32 vic_scratch32(const BlockDev& B,
                                                      const VicScratch& S,
                                                      int n) {
  VicScratch32 t;
  const size_t c = S.cells;
  float* f = reinterpret_cast<float*>(B.vic + (size_t)kVicDoublesPerCell * c);
  t.ncol = c / n;
  t.A = f;
  t.B = f + kBlk32 * c;
  t.C = f + 2 * kBlk32 * c;
  t.LU = f + 3 * kBlk32 * c;
  t.CP = t.LU + kLu32 * c;
  t.R = t.CP + kBlk32 * c;
  t.stat = t.R + kR32 * c;
  t.mask = reinterpret_cast<int*>(t.stat + 6 * t.ncol);
  return t;
}

// the padded (x3, x2) row of interior column `col` (x2 fastest)
__device__ __forceinline__ size_t vic_row(const BlockDev& B, size_t col) {
  const int ng = B.ng;
  const size_t nx2 = B.nc2 > 1 ? B.nc2 - 2 * ng : 1;
  const size_t j = col % nx2, k = col / nx2;
  return (B.nc3 > 1 ? k + ng : 0) * B.nc2 + (B.nc2 > 1 ? j + ng : 0);
}

// bit of the per-block status word: a column's solve failed this step
constexpr int kVicFailed = 32;

// a column left to the FP64 solve: the running count and the step's
// monitor count (implicit.fp64_columns)
__device__ __forceinline__ void count_fp64_column(const StageParams& p, int b) {
  atomicAdd(&p.fallbacks[b], 1ull);
  if (p.counts) atomicAdd(&p.counts[b * kCountSlots + kCountFp64Columns], 1ull);
}

template <typename T>
__device__ __forceinline__ void vmat_mul(const T* a, const T* b,
                                         T* out) {
#pragma unroll
  for (int r = 0; r < 5; ++r)
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      T s = a[r * 5] * b[c];
#pragma unroll
      for (int k = 1; k < 5; ++k) s += a[r * 5 + k] * b[k * 5 + c];
      out[r * 5 + c] = s;
    }
}

template <typename T>
__device__ __forceinline__ void vflux_jacobian(T* J, T gm1,
                                               const T* w) {
  T v1 = w[1], v2 = w[2], v3 = w[3], rho = w[0], pres = w[4];
  T s2 = v1 * v1 + v2 * v2 + v3 * v3;
  T c1 = ((gm1 - 1) * s2 / 2 - (gm1 + 1) / gm1 * pres / rho) * v1;
  T c2 = (gm1 + 1) / gm1 * pres / rho + s2 / 2 - gm1 * v1 * v1;
  J[0] = 0; J[1] = T(1.); J[2] = T(0.); J[3] = T(0.); J[4] = T(0.);
  J[5] = gm1 * s2 / 2 - v1 * v1; J[6] = (T(2.) - gm1) * v1; J[7] = -gm1 * v2;
  J[8] = -gm1 * v3; J[9] = gm1;
  J[10] = -v1 * v2; J[11] = v2; J[12] = v1; J[13] = T(0.); J[14] = T(0.);
  J[15] = -v1 * v3; J[16] = v3; J[17] = T(0.); J[18] = v1; J[19] = T(0.);
  J[20] = c1; J[21] = c2; J[22] = -gm1 * v2 * v1; J[23] = -gm1 * v3 * v1;
  J[24] = (gm1 + 1) * v1;
}

// |A| = R |Lambda| R^-1 at the face between wl and wr (Roe average)
template <typename T>
__device__ __forceinline__ void vabs_jacobian(T* A, T gm1,
                                              const T* wl,
                                              const T* wr) {
  // every quotient as written below; those sharing a divisor divide by
  // its reciprocal (vdiv: the same bits), and 1 / (2 hp), -1 / hp are the
  // reciprocals themselves
  const T gp1 = gm1 + T(1.), rgm1 = T(1.) / gm1, rgp1 = T(1.) / gp1;
  T sqrtdl = sqrt(wl[0]), sqrtdr = sqrt(wr[0]);
  T isdlpdr = T(1.0) / (sqrtdl + sqrtdr);
  T pr[5];
  pr[0] = sqrtdl * sqrtdr;
  pr[1] = (sqrtdl * wl[1] + sqrtdr * wr[1]) * isdlpdr;
  pr[2] = (sqrtdl * wl[2] + sqrtdr * wr[2]) * isdlpdr;
  pr[3] = (sqrtdl * wl[3] + sqrtdr * wr[3]) * isdlpdr;
  T el = vdiv(wl[4], gm1, rgm1) +
              T(0.5) * wl[0] * (wl[1] * wl[1] + wl[2] * wl[2] + wl[3] * wl[3]);
  T er = vdiv(wr[4], gm1, rgm1) +
              T(0.5) * wr[0] * (wr[1] * wr[1] + wr[2] * wr[2] + wr[3] * wr[3]);
  T hbar = ((el + wl[4]) / sqrtdl + (er + wr[4]) / sqrtdr) * isdlpdr;
  pr[4] = vdiv((hbar - T(0.5) * (pr[1] * pr[1] + pr[2] * pr[2] + pr[3] * pr[3])) *
                   gm1, gp1, rgp1) * pr[0];
  const T rr = T(1.) / pr[0];
  T cs = sqrt(vdiv(pr[4] * gp1, pr[0], rr));
  T r = pr[0], u = pr[1], v = pr[2], w = pr[3], p = pr[4];
  T lam[5] = {fabs(u - cs), fabs(u), fabs(u + cs), fabs(u), fabs(u)};
  T ke = T(0.5) * (u * u + v * v + w * w);
  T hp = vdiv(vdiv(gp1, gm1, rgm1) * p, r, rr);
  T h = hp + ke;
  const T d1 = T(2.) * cs * hp, d2 = T(2.) * hp;
  const T r1 = T(1.) / d1, r2 = T(1.) / d2, rh = T(1.) / hp;
  const T R[25] = {T(1.),         T(1.), T(1.),         T(0.), T(0.),  //
                        u - cs,     u,  u + cs,     T(0.), T(0.),  //
                        v,          v,  v,          T(1.), T(0.),  //
                        w,          w,  w,          T(0.), T(1.),  //
                        h - u * cs, ke, h + u * cs, v,  w};
  const T Ri[25] = {vdiv(cs * ke + u * hp, d1, r1),
                         vdiv(-hp - cs * u, d1, r1),
                         vdiv(-v, d2, r2),
                         vdiv(-w, d2, r2),
                         r2,
                         vdiv(hp - ke, hp, rh),
                         vdiv(u, hp, rh),
                         vdiv(v, hp, rh),
                         vdiv(w, hp, rh),
                         -rh,
                         vdiv(cs * ke - u * hp, d1, r1),
                         vdiv(hp - cs * u, d1, r1),
                         vdiv(-v, d2, r2),
                         vdiv(-w, d2, r2),
                         r2,
                         -v, T(0.), T(1.), T(0.), T(0.),
                         -w, T(0.), T(0.), T(1.), T(0.)};
  T RL[25];
#pragma unroll
  for (int i = 0; i < 5; ++i)
#pragma unroll
    for (int k = 0; k < 5; ++k) RL[i * 5 + k] = R[i * 5 + k] * lam[k];
  vmat_mul(RL, Ri, A);
}

// the primitives of a cell (u of the storage type -> FP64 W); an FP32
// block under gravity stores anomalies, to which the base's FP64 totals
// are added first (base null: u holds totals)
__device__ __forceinline__ void vic_prim(const real* u, size_t plane,
                                         size_t cell, double gammad,
                                         double* w, const double* base = nullptr,
                                         int nc1 = 0) {
  double uc[NHYDRO];
#pragma unroll
  for (int v = 0; v < NHYDRO; ++v) uc[v] = as_f64(u[v * plane + cell]);
  if (base) {
    const int i = (int)(cell % nc1);
    uc[IDN] = base_rho(base, nc1)[i] + uc[IDN];
    uc[IPR] = base_e(base, nc1)[i] + uc[IPR];
  }
  cons2prim<double>(uc, w, gammad);
}

// the same primitives in FP32 (FP32 assembly): the state in FP32, the base
// rounded to FP32 and added to the anomaly in FP32
__device__ __forceinline__ void vic_prim32(const real* u, size_t plane,
                                           size_t cell, float gammad,
                                           float* w, const double* base,
                                           int nc1) {
  float uc[NHYDRO];
#pragma unroll
  for (int v = 0; v < NHYDRO; ++v) uc[v] = (float)u[v * plane + cell];
  if (base) {
    const int i = (int)(cell % nc1);
    uc[IDN] = narrow_exact(base_rho(base, nc1)[i]) + uc[IDN];
    uc[IPR] = narrow_exact(base_e(base, nc1)[i]) + uc[IPR];
  }
  cons2prim<float>(uc, w, gammad);
}

// the corrected-PE slope weights of layer k of n (centres x)
// the same weights from the block's x1 geometry table (computed once, with
// these operations)
__device__ __forceinline__ void vic_slope_tab(const BlockDev& B, int n, int k,
                                              double* wt, int* i0) {
  const double* t = B.x1tab + 6 * k;
  wt[0] = t[0];
  wt[1] = t[1];
  wt[2] = t[2];
  int kc = k < 1 ? 1 : (k > n - 2 ? n - 2 : k);
  *i0 = kc - 1;
}


// the K rows of layer k: mid, lo, hi bands and the wall third points
struct VicK {
  double mid, lo, hi, t0, t1, gv;
};

__device__ __forceinline__ VicK vic_krows(const BlockDev& B, int n, int k) {
  VicK K;
  double wt[3];
  int i0;
  vic_slope_tab(B, n, k, wt, &i0);
  double gv = B.x1tab[6 * k + 3];  // grav1 h^2 / 12
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
// the blocks of interior cell e (column e / n, layer e % n) in the compute
// type T: double, or float under implicit-precision float32 (the FP32
// state's blocks, exact in FP32 and in the FP64 copies the residuals of the
// refined solve read).  The FP64 instantiation performs the reference's
// operations in its order.
// a block's constants of the assembly in the compute type, formed once per
// launch (the cell loop reloads what it reads from the block table)
template <typename T>
struct AsmConst {
  T grav, gm1, gm1r, area, vol, half_inv_vol, rvol, rdt, dtc, gammad;
  __device__ AsmConst(const BlockDev& B, double dtc_) {
    gammad = T(B.gammad);
    grav = T(B.grav1);
    gm1 = T(B.gammad - 1.);
    gm1r = T(0.5 * (B.gammad + B.gammad) - 1.);
    area = T(B.dx3 * B.dx2);
    vol = T(B.dx3 * (B.dx2 * B.dx1));
    half_inv_vol = T(0.5) / vol;
    rvol = T(1.) / vol;
    dtc = T(dtc_);
    rdt = T(1.) / dtc;
  }
};

template <typename T>
__device__ __forceinline__ void vic_assemble_cell(const BlockDev& B,
                                                  const VicScratch& S,
                                                  const real* uin,
                                                  double dtc, size_t e,
                                                  bool f32copy,
                                                  const AsmConst<T>& kc) {
  const int ng = B.ng, nc1 = B.nc1, n = nc1 - 2 * ng;
  const size_t plane = (size_t)nc1 * B.nc2 * B.nc3;
  const T grav = kc.grav, gm1 = kc.gm1;
  const T area = kc.area, vol = kc.vol;
  const double* x1v = B.x1v + ng;
  const double* x1f = B.x1f + ng;
  const bool wood = n >= 3;
  const int i = (int)(e % n);
  const size_t col = e / n;
  const size_t jrow = vic_row(B, col);
  const size_t base = jrow * nc1 + ng;  // padded cell of layer 0
  T wl[5], wr[5], wn[5];
  if constexpr (sizeof(T) == sizeof(float)) {
    // FP32 assembly: the primitives in FP32 from the FP32 state and the
    // base rounded to FP32 (the blocks are FP32 either way)
    vic_prim32(uin, plane, base + i - 1, kc.gammad, wl, B.base, nc1);
    vic_prim32(uin, plane, base + i, kc.gammad, wr, B.base, nc1);
    vic_prim32(uin, plane, base + i + 1, kc.gammad, wn, B.base, nc1);
  } else {
    double wd[3][5];
    vic_prim(uin, plane, base + i - 1, B.gammad, wd[0], B.base, nc1);
    vic_prim(uin, plane, base + i, B.gammad, wd[1], B.base, nc1);
    vic_prim(uin, plane, base + i + 1, B.gammad, wd[2], B.base, nc1);
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      wl[v] = T(wd[0][v]);
      wr[v] = T(wd[1][v]);
      wn[v] = T(wd[2][v]);
    }
  }
  T Jp[25], Jc[25], Jn[25], Am[25], Ap[25];
  const T gm1r = kc.gm1r;
  vflux_jacobian(Jp, gm1, wl);
  vflux_jacobian(Jc, gm1, wr);
  vabs_jacobian(Am, gm1r, wl, wr);
  vflux_jacobian(Jn, gm1, wn);
  vabs_jacobian(Ap, gm1r, wr, wn);
  const T half_inv_vol = kc.half_inv_vol;
  const T rvol = kc.rvol;
  const T lower = vdiv(T(0.5) * area * as_real<T>(x1v[i] - x1f[i]), vol, rvol);
  const T upper = vdiv(T(0.5) * area * as_real<T>(x1f[i + 1] - x1v[i]), vol, rvol);
  T a[25], b[25], c[25];
#pragma unroll
  for (int r = 0; r < 5; ++r)
#pragma unroll
    for (int q = 0; q < 5; ++q) {
      const int k = r * 5 + q;
      T phi = (r == 1 && q == 0) || (r == 4 && q == 1) ? grav : T(0.);
      a[k] = (Am[k] * area + Ap[k] * area + (area - area) * Jc[k]) *
                 half_inv_vol - phi;
      b[k] = -(Am[k] + Jp[k]) * area * half_inv_vol;
      c[k] = -(Ap[k] - Jn[k]) * area * half_inv_vol;
    }
  const T rdt = kc.rdt;
#pragma unroll
  for (int r = 0; r < 5; ++r) a[r * 5 + r] += rdt;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    a[20 + k] -= grav * (upper * Ap[k] - lower * Am[k]);
    b[20 + k] -= grav * lower * Am[k];
    c[20 + k] += grav * upper * Ap[k];
  }
  a[21] += grav * (T(1.) - lower - upper);
  b[21] -= grav * lower;
  c[21] -= grav * upper;
  const T bnd[5] = {T(1.), T(-1.), T(1.), T(1.), T(1.)};
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
  // the partial matrix (implicit-scheme 1, assembled in FP64 or FP32 and
  // solved in FP64 by vic_solve3_kernel): its 3x3
  // blocks are the {rho, m1, E} rows and columns of the same entries, and
  // the m_t columns of those rows (the same terms, energy-row face work and
  // wall mirror included) fold into the density column at the cell's v_t
  // and into the right-hand side at the frozen remainder
  // q_t = du[m_t] - v_t du[rho] (src/implicit/vic_assemble_impl.h:152-214);
  // the neighbours' folds are skipped at the merged walls
  const bool partial = B.implicit == 1;
  T a3[9], b3[9], c3[9], rc[3] = {T(0.), T(0.), T(0.)};
  if (partial) {
    const int rows[3] = {0, 1, 4};
    T aT[6], bT[6], cT[6];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        a3[r * 3 + q] = a[rows[r] * 5 + rows[q]];
        b3[r * 3 + q] = b[rows[r] * 5 + rows[q]];
        c3[r * 3 + q] = c[rows[r] * 5 + rows[q]];
      }
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        aT[r * 2 + k] = a[rows[r] * 5 + 2 + k];
        bT[r * 2 + k] = b[rows[r] * 5 + 2 + k];
        cT[r * 2 + k] = c[rows[r] * 5 + 2 + k];
      }
    }
    auto fold = [&](T* blk, const T* tb, int j, const T* wj) {
      const double* dj = S.du + col * n + j;  // row v at dj[v * cells]
      const T drho = T(dj[0]);
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const T v = wj[2 + k];
        const T qt = T(dj[(size_t)(2 + k) * S.cells]) - v * drho;
        if (v != T(0.))
#pragma unroll
          for (int r = 0; r < 3; ++r) blk[r * 3] = blk[r * 3] + tb[r * 2 + k] * v;
        if (qt != T(0.))
#pragma unroll
          for (int r = 0; r < 3; ++r) rc[r] = rc[r] + tb[r * 2 + k] * qt;
      }
    };
    fold(a3, aT, i, wr);
    if (i > 0) fold(b3, bT, i - 1, wl);
    if (i < n - 1) fold(c3, cT, i + 1, wn);
  }
  if (wood) {
    VicK K = vic_krows(B, n, i);
    if (partial) {
      a3[6] -= vdiv(as_real<T>(K.mid), kc.dtc, rdt);
      b3[6] -= vdiv(as_real<T>(K.lo), kc.dtc, rdt);
      c3[6] -= vdiv(as_real<T>(K.hi), kc.dtc, rdt);
    } else {
      a[20] -= vdiv(as_real<T>(K.mid), kc.dtc, rdt);
      b[20] -= vdiv(as_real<T>(K.lo), kc.dtc, rdt);
      c[20] -= vdiv(as_real<T>(K.hi), kc.dtc, rdt);
    }
    // du[IPR] -= (K du0[IDN])_i : the IDN row is read only (FP64 always)
    const double* dn = S.du + col * n;
    double s = K.mid * dn[i];
    if (i >= 1) s += K.lo * dn[i - 1];
    if (i <= n - 2) s += K.hi * dn[i + 1];
    if (i == 0) s += K.t0 * dn[2];
    if (i == n - 1) s += K.t1 * dn[n - 3];
    S.du[4 * S.cells + cell] = du0[4] - s;
  }
  if (partial) {
    // a cell's row of 25: the 3x3 block, row-major, then (A only) the
    // right-hand-side term of the fold
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      S.A[cell * 25 + k] = (double)a3[k];
      S.B[cell * 25 + k] = (double)b3[k];
      S.C[cell * 25 + k] = (double)c3[k];
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) S.A[cell * 25 + 9 + r] = (double)rc[r];
    return;
  }
  // the FP64 blocks, unless the refined solve reads the FP32 ones (exact:
  // its residuals and the masked columns' direct solve widen them)
  if (!(sizeof(T) == sizeof(float) && f32copy)) {
#pragma unroll
    for (int k = 0; k < 25; ++k) {
      S.A[cell * 25 + k] = (double)a[k];
      S.B[cell * 25 + k] = (double)b[k];
      S.C[cell * 25 + k] = (double)c[k];
    }
  }
  if (sizeof(T) == sizeof(float) && f32copy) {
    // the refined solve's FP32 sweeps read these (the same values), in
    // 16-byte stores (the row of 28 is 16-byte aligned)
    const VicScratch32 F = vic_scratch32(B, S, n);
    float4* a4 = reinterpret_cast<float4*>(F.A + cell * kBlk32);
    float4* b4 = reinterpret_cast<float4*>(F.B + cell * kBlk32);
    float4* c4 = reinterpret_cast<float4*>(F.C + cell * kBlk32);
#pragma unroll
    for (int e = 0; e < 6; ++e) {
      a4[e] = make_float4((float)a[4 * e], (float)a[4 * e + 1],
                          (float)a[4 * e + 2], (float)a[4 * e + 3]);
      b4[e] = make_float4((float)b[4 * e], (float)b[4 * e + 1],
                          (float)b[4 * e + 2], (float)b[4 * e + 3]);
      c4[e] = make_float4((float)c[4 * e], (float)c[4 * e + 1],
                          (float)c[4 * e + 2], (float)c[4 * e + 3]);
    }
    a4[6] = make_float4((float)a[24], 0.f, 0.f, 0.f);
    b4[6] = make_float4((float)b[24], 0.f, 0.f, 0.f);
    c4[6] = make_float4((float)c[24], 0.f, 0.f, 0.f);
  }
}

// CTAs of the FP32 assembly resident per SM (the register budget it is held
// to: 65536 / (256 kAsm32Ctas))
#ifndef SG_ASM32_CTAS
#define SG_ASM32_CTAS 2
#endif
constexpr int kAsm32Ctas = SG_ASM32_CTAS;

// the assembly in the compute type T: the FP64 and FP32 forms are separate
// kernels, so the FP32 one is not held to the FP64 one's register count
template <typename T>
__global__ void __launch_bounds__(kThreads, sizeof(T) == sizeof(float) ? kAsm32Ctas : 1)
    vic_assemble_kernel(const BlockDev* __restrict__ tab, StageParams p) {
  const BlockDev& B = tab[blockIdx.y];
  if (!B.implicit || (B.implicit_f32 != 0) != (sizeof(T) == sizeof(float)))
    return;
  const VicScratch S = vic_scratch(B);
  const real* uin = static_cast<const real*>(B.buf[p.in]);
  const double dtc = p.w2 * p.dt[blockIdx.y];
  const AsmConst<T> kc(B, dtc);
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < S.cells;
       e += (size_t)gridDim.x * blockDim.x)
    vic_assemble_cell<T>(B, S, uin, dtc, e, sizeof(T) == sizeof(float) && p.refine != 0,
                         kc);
}

// ludcmp<double, 5, Implicit> on a row-major 5x5 in shared memory
// (src/math/ludcmp.h); one lane runs it
// ---------------------------------------------------------------------------
// (2) the block-Thomas sweep, back substitution and Woodbury update.
//
// GB300 issues one FP64 warp instruction per SM every 16 cycles however many
// lanes it carries, so the solve packs kVicCols columns into each warp with
// kVicLanes lanes per column, and gives every lane work in every FP64
// instruction: lane q of a column owns right-hand-side column q of the
// layer's system  lu [a' | d' | z0' | z1'] = [c | rhs | e0 | e1]  (q < 5: the
// columns of c and a'; 5: d; 6, 7: the Woodbury vectors), and during the
// factorisation column q of the block (q < 5).
//
// The LU is the reference's scaled partial-pivot Crout factorisation
// (src/math/ludcmp.h) run column-per-lane in right-looking order: at step j
// the pivot column's lane picks the pivot, every lane swaps its own column's
// rows, and the later columns subtract L[i][j] U[j][c].  Each entry receives
// exactly the Crout subtractions, k ascending, so the factors are bit for
// bit the sequential ones; the failure screens of ludcmp (non-finite sums,
// zero rows, the pivot tolerance) are evaluated on the same values and any
// failure fails the column, as in the reference.  The back-solve is lubksb
// (src/math/lubksb.h) per lane: its row exchanges touch only rows not yet
// reduced, so they are applied first.
constexpr int kVicCols = 4;   // columns per warp (one warp per CTA)
constexpr int kVicLanes = 8;  // lanes per column

// a group-wide AND over the kVicLanes lanes of this lane's column
__device__ __forceinline__ bool vgroup_all(bool v, int g) {
  unsigned bad = __ballot_sync(0xffffffffu, !v);
  return ((bad >> (kVicLanes * g)) & 0xffu) == 0u;
}

__device__ __forceinline__ double vshfl(double v, int src) {
  return __shfl_sync(0xffffffffu, v, src, kVicLanes);
}

// non-negative finite doubles order like their bit patterns
__device__ __forceinline__ unsigned long long vbits(double x) {
  return static_cast<unsigned long long>(__double_as_longlong(x));
}

// a column's work array in the finish: element i at p[i s]
struct VCol {
  double* p;
  size_t s;
  __device__ __forceinline__ double& operator[](int i) const {
    return p[(size_t)i * s];
  }
};

// finite, tested on the exponent bits (integer pipes, not the FP64 one)
__device__ __forceinline__ bool vfinite(double x) {
  return ((__double_as_longlong(x) >> 52) & 0x7ff) != 0x7ff;
}

__device__ __forceinline__ double div_rcp(double a, double b, double r) {
  return vdiv<double>(a, b, r);
}

template <typename T>
__device__ __forceinline__ T vpick5(int k, T a0, T a1, T a2, T a3, T a4) {
  return k == 0 ? a0 : k == 1 ? a1 : k == 2 ? a2 : k == 3 ? a3 : a4;
}

// step J of the factorisation on this lane's column x (lanes q < 5 hold the
// block's columns; vv, scale and indx are per-lane copies of the row data)
template <int J>
__device__ __forceinline__ void vlu_step(double (&x)[5], double (&vv)[5],
                                         double (&scale)[5], double (&rsc)[5],
                                         int (&indx)[5], bool& good, int q,
                                         bool colane) {
  // pivot search on column J: the last row of the largest vv |a|
  unsigned long long best = 0ull;
  int imax = J;
#pragma unroll
  for (int i2 = J; i2 < 5; ++i2) {
    double dum = vv[i2] * fabs(x[i2]);
    if (q == J) good = good && vfinite(dum);
    if (vbits(dum) >= best) {
      best = vbits(dum);
      imax = i2;
    }
  }
  imax = __shfl_sync(0xffffffffu, imax, J, kVicLanes);
  indx[J] = imax;
#pragma unroll
  for (int i2 = J + 1; i2 < 5; ++i2)
    if (imax == i2) {
      if (colane) {
        double t = x[J];
        x[J] = x[i2];
        x[i2] = t;
      }
      vv[i2] = vv[J];
      double t = scale[J];
      scale[J] = scale[i2];
      scale[i2] = t;
      t = rsc[J];
      rsc[J] = rsc[i2];
      rsc[i2] = t;
    }
  if (J < 4) {
    double dinv = 1.0 / vshfl(x[J], J);
    double l[5];
#pragma unroll
    for (int i2 = J + 1; i2 < 5; ++i2) {
      l[i2] = vshfl(x[i2], J) * dinv;
      if (q == J) x[i2] = l[i2];
    }
    if (colane && q > J) {
#pragma unroll
      for (int i2 = J + 1; i2 < 5; ++i2) x[i2] = x[i2] - l[i2] * x[J];
    }
  }
}

struct VicSolveSmem {
  double lu[kVicCols][25];         // the factorised block of each column
  double vec[kVicCols][2][15];     // back substitution: d, z0, z1 of a layer
  double rd[kVicCols][5];          // 1 / the diagonal of each factorisation
};

// BLK32: the refined solve's masked columns, whose blocks are the FP32 ones
// (a separate instantiation, so the direct solve's block loads carry no
// select)
template <bool BLK32>
__global__ void __launch_bounds__(32)
    vic_solve_kernel(const BlockDev* __restrict__ tab, StageParams p,
                     int* status) {
  __shared__ VicSolveSmem sm;
  const BlockDev& Bk = tab[blockIdx.y];
  if (!Bk.implicit || Bk.implicit == 1) return;  // scheme 1: vic_solve3
  const VicScratch S = vic_scratch(Bk);
  const int n = Bk.nc1 - 2 * Bk.ng;
  const size_t ncol = S.cells / n;
  if ((size_t)blockIdx.x * kVicCols >= ncol) return;  // the whole warp
  const int lane = threadIdx.x, g = lane / kVicLanes, q = lane % kVicLanes;
  const size_t col = (size_t)blockIdx.x * kVicCols + g;
  bool valid = col < ncol;
  // an implicit-precision float32 block solves here only the columns its
  // refined solve left to FP64 (the mask); a warp with none leaves at once
  if (BLK32 && Bk.implicit_f32) {
    const VicScratch32 F = vic_scratch32(Bk, S, n);
    const int mk = valid ? F.mask[col] : 0;
    valid = valid && (mk == 1 || mk == 2);
    if (!__any_sync(0xffffffffu, valid)) return;
    // mask 2: the partitioned FP64 solve took the column first and
    // counted it
    if (valid && mk == 1 && q == 0) count_fp64_column(p, blockIdx.y);
  }
  // an FP64-assembled block with the partitioned form (vic_psolve_kernel,
  // which ran first): only the columns it marked
  if (Bk.psw && !Bk.implicit_f32) {
    const int* mask =
        reinterpret_cast<const int*>(Bk.psw + kPswDoublesPerCell * S.cells);
    valid = valid && mask[col < ncol ? col : ncol - 1] != 0;
    if (!__any_sync(0xffffffffu, valid)) return;
  }
  // a group past the last column (or unmasked) shadows a column and never
  // stores
  const size_t cc = col < ncol ? col : ncol - 1;
  const double dtc = p.w2 * p.dt[blockIdx.y];
  const double rdtc = 1.0 / dtc;  // every du / dt_corr divides by it
  const bool wood = n >= 3;
  const int m = wood ? 8 : 6;  // right-hand sides in use
  double* A = S.A + cc * n * 25;
  const double* Bm = S.B + cc * n * 25;
  const double* C = S.C + cc * n * 25;
  // the refined solve's masked columns: the blocks are the FP32 ones
  // (assembled in FP32, exact), widened; a' still goes to the FP64 A
  const bool blk32 = BLK32 && Bk.implicit_f32;
  const int bst = blk32 ? kBlk32 : 25;  // the row of a cell's block
  const float* A32 = nullptr;
  const float* B32 = nullptr;
  const float* C32 = nullptr;
  if (blk32) {
    const VicScratch32 F32 = vic_scratch32(Bk, S, n);
    A32 = F32.A + cc * n * kBlk32;
    B32 = F32.B + cc * n * kBlk32;
    C32 = F32.C + cc * n * kBlk32;
  }
  auto blkA = [&](int e) -> double { return blk32 ? widen_exact(A32[e]) : A[e]; };
  auto blkB = [&](int e) -> double { return blk32 ? widen_exact(B32[e]) : Bm[e]; };
  auto blkC = [&](int e) -> double { return blk32 ? widen_exact(C32[e]) : C[e]; };
  double* D = S.D + cc * n * 5;
  double* Z0 = S.Z0 + cc * n * 5;
  double* Z1 = S.Z1 + cc * n * 5;
  const double* du = S.du + cc * n;  // row v at du[v * cells + i]
  double* vout = q == 5 ? D : (q == 6 ? Z0 : Z1);
  const unsigned full = 0xffffffffu;

  // the input screen: du of every layer finite
  bool fin = true;
  for (int e = q; e < 5 * n; e += kVicLanes)
    fin = fin && vfinite(du[(size_t)(e / n) * S.cells + (e % n)]);
  // every ballot runs on all 32 lanes: evaluate before combining
  const bool fin_all = vgroup_all(fin, g);
  bool ok = valid && fin_all;

  double s[5];   // this lane's solution column of the previous layer
  double b[25];  // the b block of the layer (loaded one layer ahead)
#pragma unroll
  for (int k = 0; k < 5; ++k) s[k] = 0.;
#pragma unroll
  for (int e = 0; e < 25; ++e) b[e] = blkB(e);
  for (int i = 0; i < n; ++i) {
    if (!__any_sync(full, ok)) break;
    // this lane's column of a (q < 5), of c, and the right-hand sides
    double x[5], c5[5];
    if (q < 5) {
#pragma unroll
      for (int r = 0; r < 5; ++r) {
        x[r] = blkA(i * bst + r * 5 + q);
        c5[r] = blkC(i * bst + r * 5 + q);
      }
    } else {
#pragma unroll
      for (int r = 0; r < 5; ++r) {
        x[r] = (r == 4 && ((q == 6 && i == 0) || (q == 7 && i == n - 1))) ? 1.
                                                                         : 0.;
        c5[r] = 0.;
      }
    }
    // du / dt_corr, one row per lane, gathered on lane 5
    double dq = q < 5 ? div_rcp(du[(size_t)q * S.cells + i], dtc, rdtc) : 0.;
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      double v = vshfl(dq, r);
      if (q == 5) x[r] = v;
    }
    // x -= b s'  (a[i] - b[i] a'[i-1] and rhs - b[i] d'[i-1]), k in order
    if (i > 0) {
#pragma unroll
      for (int r = 0; r < 5; ++r) {
        double t = b[r * 5] * s[0];
#pragma unroll
        for (int k = 1; k < 5; ++k) t = t + b[r * 5 + k] * s[k];
        x[r] = x[r] - t;
      }
    }
    if (i + 1 < n) {
#pragma unroll
      for (int e = 0; e < 25; ++e) b[e] = blkB((i + 1) * bst + e);
    }

    // ---- the factorisation (lanes q < 5 hold the columns) ----
    bool good = true;
    const bool colane = q < 5;
    unsigned long long mx[5];
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      if (colane) good = good && vfinite(x[r]);
      mx[r] = colane ? vbits(fabs(x[r])) : 0ull;
    }
#pragma unroll
    for (int off = 4; off >= 1; off >>= 1)
#pragma unroll
      for (int r = 0; r < 5; ++r) {
        unsigned long long o = __shfl_xor_sync(full, mx[r], off, kVicLanes);
        mx[r] = o > mx[r] ? o : mx[r];
      }
    double scale[5], vv[5], rsc[5];
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      scale[r] = __longlong_as_double(static_cast<long long>(mx[r]));
      good = good && mx[r] != 0ull;
    }
    {
      double big = vpick5(q < 5 ? q : 0, scale[0], scale[1], scale[2],
                          scale[3], scale[4]);
      double inv = 1.0 / big;
#pragma unroll
      for (int r = 0; r < 5; ++r) vv[r] = rsc[r] = vshfl(inv, r);
    }
#pragma unroll
    for (int r = 0; r < 5; ++r) good = good && vfinite(vv[r]);
    int indx[5];
    vlu_step<0>(x, vv, scale, rsc, indx, good, q, colane);
    vlu_step<1>(x, vv, scale, rsc, indx, good, q, colane);
    vlu_step<2>(x, vv, scale, rsc, indx, good, q, colane);
    vlu_step<3>(x, vv, scale, rsc, indx, good, q, colane);
    vlu_step<4>(x, vv, scale, rsc, indx, good, q, colane);
    if (colane) {
#pragma unroll
      for (int r = 0; r < 5; ++r) good = good && vfinite(x[r]);
      // the pivot tolerance of every step, on the final diagonal and scale
      // (|d| / scale, from the scale's reciprocal carried through the swaps)
      double dg = vpick5(q, x[0], x[1], x[2], x[3], x[4]);
      double sc = vpick5(q, scale[0], scale[1], scale[2], scale[3], scale[4]);
      double rs = vpick5(q, rsc[0], rsc[1], rsc[2], rsc[3], rsc[4]);
      good = good && !(div_rcp(fabs(dg), sc, rs) <= 8. * 5 * 2.220446049250313e-16);
      // stage the factors, and the diagonal's reciprocals, for every lane's
      // back-solve
#pragma unroll
      for (int r = 0; r < 5; ++r) sm.lu[g][r * 5 + q] = x[r];
      sm.rd[g][q] = 1.0 / dg;
    }
    const bool good_all = vgroup_all(good, g);
    ok = ok && good_all;
    __syncwarp();

    // ---- lubksb on this lane's right-hand side ----
    double sol[5];
#pragma unroll
    for (int r = 0; r < 5; ++r) sol[r] = colane ? c5[r] : x[r];
#pragma unroll
    for (int rr = 0; rr < 5; ++rr) {
      const int ip = indx[rr];
#pragma unroll
      for (int k = rr + 1; k < 5; ++k)
        if (ip == k) {
          double t = sol[k];
          sol[k] = sol[rr];
          sol[rr] = t;
        }
    }
    const double* lu = sm.lu[g];
#pragma unroll
    for (int rr = 1; rr < 5; ++rr)
#pragma unroll
      for (int jj = 0; jj < rr; ++jj) sol[rr] = sol[rr] - lu[rr * 5 + jj] * sol[jj];
#pragma unroll
    for (int rr = 4; rr >= 0; --rr) {
#pragma unroll
      for (int jj = rr + 1; jj < 5; ++jj)
        sol[rr] = sol[rr] - lu[rr * 5 + jj] * sol[jj];
      sol[rr] = div_rcp(sol[rr], lu[rr * 5 + rr], sm.rd[g][rr]);
    }
    bool f = true;
    if (q < m) {
#pragma unroll
      for (int r = 0; r < 5; ++r) f = f && vfinite(sol[r]);
    }
    const bool f_all = vgroup_all(f, g);
    ok = ok && f_all;
    if (valid) {
      if (colane) {
#pragma unroll
        for (int r = 0; r < 5; ++r) A[i * 25 + r * 5 + q] = sol[r];
      } else if (q < m) {
#pragma unroll
        for (int r = 0; r < 5; ++r) vout[i * 5 + r] = sol[r];
      }
    }
#pragma unroll
    for (int r = 0; r < 5; ++r) s[r] = sol[r];
    __syncwarp();
  }

  // ---- back substitution: x[i] -= a'[i] x[i+1] for d, z0, z1 ----
  // lane q handles the (vector, row) pairs q and q + 8 of the 15
  if (__any_sync(full, ok)) {
    if (q >= 5) {
#pragma unroll
      for (int r = 0; r < 5; ++r) sm.vec[g][0][(q - 5) * 5 + r] = s[r];
    }
    __syncwarp();
    int cur = 0;
    for (int i = n - 2; i >= 0; --i) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int pr = q + kVicLanes * h;
        if (pr < 15) {
          const int v = pr / 5, r = pr % 5;
          const double* xn = sm.vec[g][cur] + v * 5;
          const double* ar = A + i * 25 + r * 5;
          double t = ar[0] * xn[0];
#pragma unroll
          for (int k = 1; k < 5; ++k) t = t + ar[k] * xn[k];
          double* vec = v == 0 ? D : (v == 1 ? Z0 : Z1);
          double val = vec[i * 5 + r] - t;
          if (ok) vec[i * 5 + r] = val;
          sm.vec[g][cur ^ 1][pr] = val;
        }
      }
      __syncwarp();
      cur ^= 1;
    }
    if (wood && ok) {
      VicK K0 = vic_krows(Bk, n, 0), K1 = vic_krows(Bk, n, n - 1);
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
      // this column's lanes (ok and wood are uniform over them) finish
      // reading D and Z before any of them updates D
      __syncwarp(0xffu << (kVicLanes * g));
      for (int e = q; e < 5 * n; e += kVicLanes) {
        double d = D[e];
        d -= Z0[e] * al0;
        d -= Z1[e] * al1;
        D[e] = d;
      }
    }
    __syncwarp();
    bool f = true;
    if (ok)
      for (int e = q; e < 5 * n; e += kVicLanes) f = f && vfinite(D[e]);
    const bool d_all = vgroup_all(f, g);
    ok = ok && d_all;
  }
  // a failed column is marked in its solution: the finish keeps du0
  if (valid && !ok && q == 0) {
    D[0] = __longlong_as_double(0x7ff8000000000000ll);
    atomicOr(&status[blockIdx.y], kVicFailed);
  }
}

// ---------------------------------------------------------------------------
// (2p) the partial matrix (implicit-scheme 1): the 3x3 block-Thomas sweep of
// ForwardSweep with N = 3 (src/implicit/forward_sweep_impl.h:30-131), one
// thread per column: the right-hand side less the assembly's fold term, the
// block screened by ludcmp<3> and inverted explicitly (adjugate over the
// determinant), d = inv (rhs - b d_prev), a' = inv c, the two Woodbury unit
// vectors of the energy row, then vic_backward_substitute (each vector only
// if its first layer is finite) and the Woodbury update on the 3-vectors.
// The solution leaves in D rows 0, 1 and 4 (the tangential rows keep the
// explicit du; the finish moves them with the face mass).  Its chain is
// short (about 200 FP64 operations per layer), so a thread per column keeps
// every lane of an FP64 instruction on its own column.
__device__ __forceinline__ bool vic_ludcmp3_ok(const double* m) {
  double a[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    a[k] = m[k];
    if (!vfinite(a[k])) return false;
  }
  double vv[3], scale[3];
  const double tol = 8. * 3 * 2.220446049250313e-16;
  for (int i = 0; i < 3; ++i) {
    double big = 0.;
    for (int j = 0; j < 3; ++j) {
      const double t = fabs(a[i * 3 + j]);
      if (t > big) big = t;
    }
    if (big == 0.) return false;
    scale[i] = big;
    vv[i] = 1.0 / big;
    if (!vfinite(vv[i])) return false;
  }
  for (int j = 0; j < 3; ++j) {
    for (int i = 0; i < j; ++i) {
      double sum = a[i * 3 + j];
      for (int k = 0; k < i; ++k) sum -= a[i * 3 + k] * a[k * 3 + j];
      if (!vfinite(sum)) return false;
      a[i * 3 + j] = sum;
    }
    double big = 0.;
    int imax = 0;
    for (int i = j; i < 3; ++i) {
      double sum = a[i * 3 + j];
      for (int k = 0; k < j; ++k) sum -= a[i * 3 + k] * a[k * 3 + j];
      if (!vfinite(sum)) return false;
      a[i * 3 + j] = sum;
      const double dum = vv[i] * fabs(sum);
      if (!vfinite(dum)) return false;
      if (dum >= big) {
        big = dum;
        imax = i;
      }
    }
    if (j != imax) {
      for (int k = 0; k < 3; ++k) {
        const double t = a[imax * 3 + k];
        a[imax * 3 + k] = a[j * 3 + k];
        a[j * 3 + k] = t;
      }
      vv[imax] = vv[j];
      const double t = scale[imax];
      scale[imax] = scale[j];
      scale[j] = t;
    }
    if (fabs(a[j * 3 + j]) / scale[j] <= tol) return false;
    if (j != 2) {
      const double dum = 1.0 / a[j * 3 + j];
      for (int i = j + 1; i < 3; ++i) a[i * 3 + j] *= dum;
    }
  }
#pragma unroll
  for (int k = 0; k < 9; ++k)
    if (!vfinite(a[k])) return false;
  return true;
}

__device__ __forceinline__ void vmat3_mul(double* out, const double* a,
                                          const double* b) {
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      double s = a[r * 3] * b[c];
      s += a[r * 3 + 1] * b[3 + c];
      s += a[r * 3 + 2] * b[6 + c];
      out[r * 3 + c] = s;
    }
}

__device__ __forceinline__ void vmat3_vec(double* out, const double* a,
                                          const double* v) {
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    double s = a[r * 3] * v[0];
    s += a[r * 3 + 1] * v[1];
    s += a[r * 3 + 2] * v[2];
    out[r] = s;
  }
}

__global__ void __launch_bounds__(kThreads)
    vic_solve3_kernel(const BlockDev* __restrict__ tab, StageParams p,
                      int* status) {
  const BlockDev& Bk = tab[blockIdx.y];
  if (Bk.implicit != 1) return;
  const VicScratch S = vic_scratch(Bk);
  const int n = Bk.nc1 - 2 * Bk.ng;
  const size_t ncol = S.cells / n;
  const size_t col = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const double dtc = p.w2 * p.dt[blockIdx.y];
  const double rdtc = 1. / dtc;  // du / dt_corr divides by it (vdiv)
  const bool wood = n >= 3;
  double* A = S.A + col * n * 25;
  const double* Bm = S.B + col * n * 25;
  const double* C = S.C + col * n * 25;
  double* D = S.D + col * n * 5;
  double* Z0 = S.Z0 + col * n * 5;
  double* Z1 = S.Z1 + col * n * 5;
  const double* du = S.du + col * n;  // row v at du[v * cells + i]
  const size_t cs = S.cells;
  bool ok = true;
  for (int e = 0; e < 5 * n; ++e)
    ok = ok && vfinite(du[(size_t)(e / n) * cs + (e % n)]);
  double ap[9], dp[3], y0[3] = {0., 0., 0.}, y1[3] = {0., 0., 0.};
  for (int i = 0; i < n && ok; ++i) {
    double m[9], bb[9], cc[9], rc[3];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      m[k] = A[i * 25 + k];
      bb[k] = Bm[i * 25 + k];
      cc[k] = C[i * 25 + k];
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) rc[r] = A[i * 25 + 9 + r];
    double rhs[3] = {vdiv(du[i], dtc, rdtc), vdiv(du[cs + i], dtc, rdtc),
                     vdiv(du[4 * cs + i], dtc, rdtc)};
#pragma unroll
    for (int r = 0; r < 3; ++r)
      if (rc[r] != 0.) rhs[r] -= rc[r];
    if (i > 0) {
      double t[9];
      vmat3_mul(t, bb, ap);
#pragma unroll
      for (int k = 0; k < 9; ++k) m[k] -= t[k];
    }
    if (!vic_ludcmp3_ok(m)) {
      ok = false;
      break;
    }
    // the adjugate over the determinant, expanded along column 0
    const double c00 = m[4] * m[8] - m[5] * m[7];
    const double c10 = m[2] * m[7] - m[1] * m[8];
    const double c20 = m[1] * m[5] - m[2] * m[4];
    const double det = m[0] * c00 + m[3] * c10 + m[6] * c20;
    const double rd = 1. / det;
    const double inv[9] = {c00 * rd,
                           c10 * rd,
                           c20 * rd,
                           (m[5] * m[6] - m[3] * m[8]) * rd,
                           (m[0] * m[8] - m[2] * m[6]) * rd,
                           (m[2] * m[3] - m[0] * m[5]) * rd,
                           (m[3] * m[7] - m[4] * m[6]) * rd,
                           (m[1] * m[6] - m[0] * m[7]) * rd,
                           (m[0] * m[4] - m[1] * m[3]) * rd};
    double t[3], u[3];
    if (i > 0) {
      vmat3_vec(u, bb, dp);
#pragma unroll
      for (int r = 0; r < 3; ++r) t[r] = rhs[r] - u[r];
    } else {
#pragma unroll
      for (int r = 0; r < 3; ++r) t[r] = rhs[r];
    }
    vmat3_vec(dp, inv, t);
    if (wood) {
      if (i > 0) {
        vmat3_vec(u, bb, y0);
#pragma unroll
        for (int r = 0; r < 3; ++r) t[r] = (r == 2 && i == 0 ? 1. : 0.) - u[r];
      } else {
        t[0] = 0.;
        t[1] = 0.;
        t[2] = 1.;
      }
      vmat3_vec(y0, inv, t);
      if (i > 0) {
        vmat3_vec(u, bb, y1);
#pragma unroll
        for (int r = 0; r < 3; ++r) t[r] = (r == 2 && i == n - 1 ? 1. : 0.) - u[r];
      } else {
        t[0] = 0.;
        t[1] = 0.;
        t[2] = i == n - 1 ? 1. : 0.;
      }
      vmat3_vec(y1, inv, t);
    }
    vmat3_mul(ap, inv, cc);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      ok = ok && vfinite(dp[r]);
#pragma unroll
      for (int q = 0; q < 3; ++q) ok = ok && vfinite(ap[r * 3 + q]);
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) A[i * 25 + k] = ap[k];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      D[i * 5 + r] = dp[r];
      Z0[i * 5 + r] = y0[r];
      Z1[i * 5 + r] = y1[r];
    }
  }
  if (ok) {
    bool f0 = wood, f1 = wood;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      f0 = f0 && vfinite(Z0[r]);
      f1 = f1 && vfinite(Z1[r]);
    }
    for (int i = n - 2; i >= 0; --i) {
      double a[9], t[3];
#pragma unroll
      for (int k = 0; k < 9; ++k) a[k] = A[i * 25 + k];
      vmat3_vec(t, a, dp);
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        dp[r] = D[i * 5 + r] - t[r];
        D[i * 5 + r] = dp[r];
      }
      if (f0) {
        vmat3_vec(t, a, y0);
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          y0[r] = Z0[i * 5 + r] - t[r];
          Z0[i * 5 + r] = y0[r];
        }
      }
      if (f1) {
        vmat3_vec(t, a, y1);
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          y1[r] = Z1[i * 5 + r] - t[r];
          Z1[i * 5 + r] = y1[r];
        }
      }
    }
    double al0 = 0., al1 = 0.;
    if (wood) {
      VicK K0 = vic_krows(Bk, n, 0), K1 = vic_krows(Bk, n, n - 1);
      double k0 = -K0.t0 / dtc, k1 = -K1.t1 / dtc;
      k0 = k0 * 1.;
      k1 = k1 * 1.;
      const int a0 = 2, a1 = n - 3;
      double m00 = 1. + k0 * Z0[a0 * 5], m01 = k0 * Z1[a0 * 5];
      double m10 = k1 * Z0[a1 * 5], m11 = 1. + k1 * Z1[a1 * 5];
      double r0 = k0 * D[a0 * 5], r1 = k1 * D[a1 * 5];
      double det = m00 * m11 - m01 * m10;
      al0 = (m11 * r0 - m01 * r1) / det;
      al1 = (m00 * r1 - m10 * r0) / det;
    }
    for (int i = 0; i < n; ++i) {
      double d[3];
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        d[r] = D[i * 5 + r];
        if (wood) {
          d[r] -= Z0[i * 5 + r] * al0;
          d[r] -= Z1[i * 5 + r] * al1;
        }
        ok = ok && vfinite(d[r]);
      }
      D[i * 5] = d[0];
      D[i * 5 + 1] = d[1];
      D[i * 5 + 2] = 0.;
      D[i * 5 + 3] = 0.;
      D[i * 5 + 4] = d[2];
    }
  }
  // a failed column is marked in its solution: the finish keeps du0
  if (!ok) {
    D[0] = __longlong_as_double(0x7ff8000000000000ll);
    atomicOr(&status[blockIdx.y], kVicFailed);
  }
}

constexpr int kVicWarps = 4;  // columns per CTA of the finish (a warp each)

// (3) redistribution, the gravity-work remainder and the RK combine of each
// column, one warp per column: the serial passes of the constituent column
// (sums, face-mass prefix, availability clamp) on lane 0, the per-layer maps
// on every lane
template <int NL>
__device__ __forceinline__ void vsync() {
  if (NL > 1) __syncwarp();
}

// ---------------------------------------------------------------------------
// the refined solve of implicit-precision float32 blocks.  The block-
// tridiagonal system T x = b of every column (the right-hand sides du /
// dt_corr and the two Woodbury unit vectors) is solved by the block-Thomas
// sweep in FP32 (vic_solve32_kernel, the direct solve's lane layout), then
// corrected p.refine times (1 to 3): the FP64 residual r = b - T x
// (vic_residual_kernel, from the FP32-assembled blocks widened to FP64,
// which is exact) is solved by the same FP32 sweep and added to x in FP64.
// That is mixed-precision iterative refinement (the scheme of LAPACK's
// dsgesv): x converges to the FP64 solution by a factor of about
// kappa(T) eps32 per correction, the factorisation on the FP32 pipes and
// only the residuals in FP64.  The solutions accumulate in the direct
// solve's D, Z0, Z1.  A column whose FP32 factorisation fails or whose last
// correction leaves an estimated error above 2^-44 of its solution takes the
// direct FP64 solve instead (vic_solve_kernel, which reads the mask), as the
// reference retries a failed FP32 column in FP64 (src/hydro/hydro.cpp:436-
// 466).
// ---------------------------------------------------------------------------
__device__ __forceinline__ float vshfl32(float v, int src) {
  return __shfl_sync(0xffffffffu, v, src, kVicLanes);
}

__device__ __forceinline__ bool vfinite32(float x) {
  return ((__float_as_uint(x) >> 23) & 0xffu) != 0xffu;
}

// step J of the FP32 factorisation on this lane's column x (the layout of
// vlu_step: lanes q < 5 hold the block's columns, every lane keeps the row
// data); the reciprocals are correctly rounded, the rest is FP32 arithmetic
template <int J>
__device__ __forceinline__ void vlu32_step(float (&x)[5], float (&vv)[5],
                                           float (&scale)[5], int (&indx)[5],
                                           bool& good, int q, bool colane) {
  float best = -1.f;
  int imax = J;
#pragma unroll
  for (int i2 = J; i2 < 5; ++i2) {
    const float dum = vv[i2] * fabsf(x[i2]);
    if (dum >= best) {
      best = dum;
      imax = i2;
    }
  }
  imax = __shfl_sync(0xffffffffu, imax, J, kVicLanes);
  indx[J] = imax;
#pragma unroll
  for (int i2 = J + 1; i2 < 5; ++i2) {
    const bool sw = imax == i2;
    const float xj = x[J], xi = x[i2];
    if (colane) {
      x[J] = sw ? xi : xj;
      x[i2] = sw ? xj : xi;
    }
    const float vj = vv[J], vi = vv[i2];
    vv[i2] = sw ? vj : vi;
    const float sj = scale[J], si = scale[i2];
    scale[J] = sw ? si : sj;
    scale[i2] = sw ? sj : si;
  }
  if (J < 4) {
    const float piv = vshfl32(x[J], J);
    good = good && piv != 0.f;
    const float dinv = __frcp_rn(piv);
    float l[5];
#pragma unroll
    for (int i2 = J + 1; i2 < 5; ++i2) {
      l[i2] = vshfl32(x[i2], J) * dinv;
      if (q == J) x[i2] = l[i2];
    }
    if (colane && q > J) {
#pragma unroll
      for (int i2 = J + 1; i2 < 5; ++i2) x[i2] = fmaf(-l[i2], x[J], x[i2]);
    }
  }
}

struct VicSolve32Smem {
  float lu[kVicCols][25];       // the factorised block of each column
  float rd[kVicCols][5];        // 1 / the diagonal of each factorisation
  float vec[kVicCols][2][15];   // back substitution: d, z0, z1 of a layer
};

// the first, factoring pass of the refined solve, kVicCols columns per
// warp, lane q of a column owning right-hand-side column q of  lu [c' | y |
// y0 | y1] = [c | b | e0 | e1]  as in vic_solve_kernel: the block-Thomas
// sweep in FP32 for b = du / dt_corr and the unit vectors, x into D, Z0, Z1.
// It keeps each layer's LU factors (with the diagonal's reciprocals and the
// pivot rows), c' and y for the corrections, and per column the largest |x|
// of each right-hand side; a column whose factorisation fails is masked
// (held to 96 registers, 20 single-warp CTAs per SM instead of 16: the
// sweep's chain hides behind more columns; ensemble solve phase 3.53 ->
// 3.45 ms per stage)
__global__ void __launch_bounds__(32, 20)
    vic_solve32_kernel(const BlockDev* __restrict__ tab, StageParams p) {
  __shared__ VicSolve32Smem sm;
  const BlockDev& Bk = tab[blockIdx.y];
  // (scheme-9 blocks only: a scheme-1 block assembled in FP32 is solved
  // in FP64 by vic_solve3_kernel)
  if (Bk.implicit != 9 || !Bk.implicit_f32) return;
  const VicScratch S = vic_scratch(Bk);
  const int n = Bk.nc1 - 2 * Bk.ng;
  const VicScratch32 F = vic_scratch32(Bk, S, n);
  const size_t ncol = F.ncol;
  if ((size_t)blockIdx.x * kVicCols >= ncol) return;
  const int lane = threadIdx.x, g = lane / kVicLanes, q = lane % kVicLanes;
  const size_t col = (size_t)blockIdx.x * kVicCols + g;
  // a group past the last column shadows a column and never stores
  const bool valid = col < ncol;
  const size_t cc = valid ? col : ncol - 1;
  bool ok = valid;
  if (!__any_sync(0xffffffffu, ok)) return;
  const double dtc = p.w2 * p.dt[blockIdx.y];
  const bool wood = n >= 3;
  const int m = wood ? 8 : 6;  // right-hand sides in use
  const float* A = F.A + cc * n * kBlk32;
  const float* Bm = F.B + cc * n * kBlk32;
  const float* C = F.C + cc * n * kBlk32;
  float* LU = F.LU + cc * n * kLu32;
  float* CP = F.CP + cc * n * kBlk32;
  float* R = F.R + cc * n * kR32;
  const double* du = S.du + cc * n;
  const float rdtc = (float)(1. / dtc);
  const bool colane = q < 5;
  const unsigned full = 0xffffffffu;

  float s[5];  // this lane's y of the previous layer
#pragma unroll
  for (int k = 0; k < 5; ++k) s[k] = 0.f;
  {
    // ---- the forward sweep: lanes q < 5 carry the block's columns ----
    // a layer's loads, issued one layer ahead: this lane's column of a and
    // of c (q < 5), du / dt_corr of row q (q < 5) or the unit vectors, b
    float xa[5], ca[5], dqa = 0.f;
    float4 bn[kBlk32 / 4];
    auto load = [&](int i) {
#pragma unroll
      for (int r = 0; r < 5; ++r) {
        if (colane) {
          xa[r] = A[i * kBlk32 + r * 5 + q];
          ca[r] = C[i * kBlk32 + r * 5 + q];
        } else {
          xa[r] = (r == 4 && ((q == 6 && i == 0) || (q == 7 && i == n - 1)))
                      ? 1.f : 0.f;
          ca[r] = 0.f;
        }
      }
      if (colane) dqa = (float)du[(size_t)q * S.cells + i] * rdtc;
      const float4* b4 = reinterpret_cast<const float4*>(Bm + i * kBlk32);
#pragma unroll
      for (int k = 0; k < kBlk32 / 4; ++k) bn[k] = b4[k];
    };
    load(0);
    for (int i = 0; i < n; ++i) {
      if (!__any_sync(full, ok)) break;
      float x[5], c5[5], b[kBlk32];
#pragma unroll
      for (int r = 0; r < 5; ++r) {
        x[r] = xa[r];
        c5[r] = ca[r];
      }
#pragma unroll
      for (int k = 0; k < kBlk32 / 4; ++k) {
        b[4 * k] = bn[k].x;
        b[4 * k + 1] = bn[k].y;
        b[4 * k + 2] = bn[k].z;
        b[4 * k + 3] = bn[k].w;
      }
      const float dq = dqa;
      if (i + 1 < n) load(i + 1);
#pragma unroll
      for (int r = 0; r < 5; ++r) {  // du / dt_corr gathered on lane 5
        const float v = vshfl32(dq, r);
        if (q == 5) x[r] = v;
      }
      if (i > 0) {
#pragma unroll
        for (int r = 0; r < 5; ++r) {
          float t = x[r];
#pragma unroll
          for (int k = 0; k < 5; ++k) t = fmaf(-b[r * 5 + k], s[k], t);
          x[r] = t;
        }
      }
      // the factorisation, scaled partial pivoting
      bool good = true;
      unsigned mx[5];
#pragma unroll
      for (int r = 0; r < 5; ++r) {
        if (colane) good = good && vfinite32(x[r]);
        mx[r] = colane ? __float_as_uint(fabsf(x[r])) : 0u;
      }
#pragma unroll
      for (int off = 4; off >= 1; off >>= 1)
#pragma unroll
        for (int r = 0; r < 5; ++r)
          mx[r] = max(mx[r], __shfl_xor_sync(full, mx[r], off, kVicLanes));
      float scale[5], vv[5];
#pragma unroll
      for (int r = 0; r < 5; ++r) {
        scale[r] = __uint_as_float(mx[r]);
        good = good && mx[r] != 0u;
      }
      {
        const float big = vpick5(q < 5 ? q : 0, scale[0], scale[1], scale[2],
                                 scale[3], scale[4]);
        const float inv = __frcp_rn(big);
#pragma unroll
        for (int r = 0; r < 5; ++r) vv[r] = vshfl32(inv, r);
      }
      int indx[5];
      vlu32_step<0>(x, vv, scale, indx, good, q, colane);
      vlu32_step<1>(x, vv, scale, indx, good, q, colane);
      vlu32_step<2>(x, vv, scale, indx, good, q, colane);
      vlu32_step<3>(x, vv, scale, indx, good, q, colane);
      vlu32_step<4>(x, vv, scale, indx, good, q, colane);
      if (colane) {
        const float dg = vpick5(q, x[0], x[1], x[2], x[3], x[4]);
        const float sc =
            vpick5(q, scale[0], scale[1], scale[2], scale[3], scale[4]);
        // the pivot tolerance, in FP32's epsilon
        good = good && vfinite32(dg) &&
               fabsf(dg) > 8.f * 5.f * 1.1920929e-7f * sc;
        const float rdg = __frcp_rn(dg);
#pragma unroll
        for (int r = 0; r < 5; ++r) sm.lu[g][r * 5 + q] = x[r];
        sm.rd[g][q] = rdg;
        // the factors for the corrections
        if (valid) {
#pragma unroll
          for (int r = 0; r < 5; ++r) LU[i * kLu32 + r * 5 + q] = x[r];
          LU[i * kLu32 + 25 + q] = rdg;
          if (q == 0) {
            int pk = 0;
#pragma unroll
            for (int j = 0; j < 5; ++j) pk |= indx[j] << (3 * j);
            LU[i * kLu32 + 30] = __int_as_float(pk);
          }
        }
      }
      ok = ok && vgroup_all(good, g);
      __syncwarp();
      // the back-solve of this lane's right-hand side
      float sol[5];
#pragma unroll
      for (int r = 0; r < 5; ++r) sol[r] = colane ? c5[r] : x[r];
#pragma unroll
      for (int rr = 0; rr < 5; ++rr) {
        const int ip = indx[rr];
#pragma unroll
        for (int k = rr + 1; k < 5; ++k) {
          const bool sw = ip == k;
          const float a = sol[rr], c = sol[k];
          sol[rr] = sw ? c : a;
          sol[k] = sw ? a : c;
        }
      }
      const float* lu = sm.lu[g];
#pragma unroll
      for (int rr = 1; rr < 5; ++rr)
#pragma unroll
        for (int jj = 0; jj < rr; ++jj)
          sol[rr] = fmaf(-lu[rr * 5 + jj], sol[jj], sol[rr]);
#pragma unroll
      for (int rr = 4; rr >= 0; --rr) {
#pragma unroll
        for (int jj = rr + 1; jj < 5; ++jj)
          sol[rr] = fmaf(-lu[rr * 5 + jj], sol[jj], sol[rr]);
        sol[rr] = sol[rr] * sm.rd[g][rr];
      }
      if (valid) {
        if (colane) {
#pragma unroll
          for (int r = 0; r < 5; ++r) CP[i * kBlk32 + r * 5 + q] = sol[r];
        } else if (q < m) {
#pragma unroll
          for (int r = 0; r < 5; ++r) R[i * kR32 + (q - 5) * 5 + r] = sol[r];
        }
      }
#pragma unroll
      for (int r = 0; r < 5; ++r) s[r] = sol[r];
      __syncwarp();
    }
  }

  // ---- back substitution: x_i = y_i - c'_i x_(i+1), into D, Z0, Z1 ----
  // lane q handles the (vector, row) pairs q and q + 8 of the 15; a layer's
  // c' row and y are loaded a layer ahead
  float dmax[2] = {0.f, 0.f};
  bool fin = true;
  if (__any_sync(full, ok)) {
    double* const D0 = S.D + cc * n * 5;
    double* const Z0 = S.Z0 + cc * n * 5;
    double* const Z1 = S.Z1 + cc * n * 5;
    bool use[2];
    double* xp[2];
    int pr2[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int pr = q + kVicLanes * h;
      pr2[h] = pr;
      use[h] = pr < 15 && (pr < 5 || wood);
      const int v = pr / 5, r = pr % 5;
      xp[h] = (v == 0 ? D0 : (v == 1 ? Z0 : Z1)) + r;
    }
    float crn[2][5], yn[2];
    auto bload = [&](int i) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        if (use[h]) {
          const int r = pr2[h] % 5;
#pragma unroll
          for (int k = 0; k < 5; ++k) crn[h][k] = CP[i * kBlk32 + r * 5 + k];
          yn[h] = R[i * kR32 + pr2[h]];
        }
      }
    };
    if (q >= 5) {
#pragma unroll
      for (int r = 0; r < 5; ++r) sm.vec[g][0][(q - 5) * 5 + r] = s[r];
    }
    if (n >= 2) bload(n - 2);
    __syncwarp();
    // the last layer: x = y
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (use[h]) {
        const float val = sm.vec[g][0][pr2[h]];
        if (ok) xp[h][(n - 1) * 5] = widen_exact(val);
        fin = fin && vfinite32(val);
        dmax[h] = fmaxf(dmax[h], fabsf(val));
      }
    }
    int cur = 0;
    for (int i = n - 2; i >= 0; --i) {
      float cr[2][5], y[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
#pragma unroll
        for (int k = 0; k < 5; ++k) cr[h][k] = crn[h][k];
        y[h] = yn[h];
      }
      if (i > 0) bload(i - 1);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        if (use[h]) {
          const float* xn = sm.vec[g][cur] + (pr2[h] / 5) * 5;
          float t = y[h];
#pragma unroll
          for (int k = 0; k < 5; ++k) t = fmaf(-cr[h][k], xn[k], t);
          sm.vec[g][cur ^ 1][pr2[h]] = t;
          if (ok) xp[h][i * 5] = widen_exact(t);
          fin = fin && vfinite32(t);
          dmax[h] = fmaxf(dmax[h], fabsf(t));
        }
      }
      __syncwarp();
      cur ^= 1;
    }
  }
  ok = ok && vgroup_all(fin, g);
  // the largest |x| of each right-hand side over the column's lanes
  // (pairs: vector pr / 5): the solution's scale, and the first "update"
  float dv[3];
#pragma unroll
  for (int v = 0; v < 3; ++v) {
    float dl = 0.f;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int pr = q + kVicLanes * h;
      if (pr < 15 && pr / 5 == v) dl = fmaxf(dl, dmax[h]);
    }
#pragma unroll
    for (int off = 4; off >= 1; off >>= 1)
      dl = fmaxf(dl, __shfl_xor_sync(full, dl, off, kVicLanes));
    dv[v] = dl;
  }
  if (valid && ok && q < 3) {
    float* st = F.stat + cc * 6;
    const float d = vpick5(q, dv[0], dv[1], dv[2], 0.f, 0.f);
    st[q] = d;
    st[3 + q] = d;
  }
  if (valid && q == 0) F.mask[cc] = ok ? 0 : 1;
}

// a correction of the refined solve, one thread per column and right-hand
// side (kCorrCols columns of three lanes per warp, kCorrWarps warps per
// CTA): y_i = LU_i^-1 (r_i - b_i y_(i-1)) from the stored factors, then
// d_i = y_i - c'_i d_(i+1), added to x in FP64.  Each sweep runs over a
// ring of kCorrRing layers in shared memory that the warp fills with
// asynchronous copies (cp.async) kCorrRing - 1 layers ahead: a column's
// factors, b and residuals going forward, c', y and x going back.  Per
// column and right-hand side the largest |d| is kept.  The last correction
// decides convergence: the error it leaves is about |d| rho, rho = |d| /
// |d_prev| the observed contraction, accepted at or below 2^-44 of the
// largest |x|.  A converged column then gets the Woodbury step of the direct
// solve; the others are masked for the direct FP64 solve
// (one box, the same runs: 10 columns with a 6-layer ring 3.33 ms per
// stage on the ensemble, 8 with 8 layers 3.26 ms and the served trace
// +0.5 %, 6 with 8 layers 3.29 ms)
#ifndef SG_CORR_COLS
#define SG_CORR_COLS 8
#endif
#ifndef SG_CORR_RING
#define SG_CORR_RING 8
#endif
constexpr int kCorrCols = SG_CORR_COLS;  // columns per warp (3 lanes each)
// (one warp per CTA with a 6-layer ring, 20 KB: measured against two warps
// with a 4-layer ring on one box, the ensemble's solve phase 3.53 -> 3.31
// ms per stage, the served trace +0.7 %)
constexpr int kCorrWarps = 1;   // warps per CTA
constexpr int kCorrRing = SG_CORR_RING;  // layers in flight per warp
// shared-memory row strides of a column's factors and residuals: multiples
// of 4 floats (16-byte copies) that spread a warp's columns over the
// banks (at most two columns per bank)
constexpr int kLuRow = kLu32 + 4, kRRow = kR32 + 4;

union __align__(16) CorrSlot {
  struct {
    float lu[kCorrCols][kLuRow];
    float b[kCorrCols][kBlk32];
    float r[kCorrCols][kRRow];
  } f;  // forward
  struct {
    float cp[kCorrCols][kBlk32];
    float y[kCorrCols][kRRow];  // the column's y rows, as the forward r
    double x[32][5];
  } g;  // back
};

__device__ __forceinline__ void cpa16(void* s, const void* g) {
  const unsigned a = static_cast<unsigned>(__cvta_generic_to_shared(s));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(a), "l"(g)
               : "memory");
}
__device__ __forceinline__ void cpa8(void* s, const void* g) {
  const unsigned a = static_cast<unsigned>(__cvta_generic_to_shared(s));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(a), "l"(g)
               : "memory");
}
__device__ __forceinline__ void cpa_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
// this thread's copies of all but the newest n groups are complete
template <int N>
__device__ __forceinline__ void cpa_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

__global__ void __launch_bounds__(32 * kCorrWarps)
    vic_correct32_kernel(const BlockDev* __restrict__ tab, StageParams p,
                         int last) {
  __shared__ CorrSlot ring[kCorrWarps][kCorrRing];
  const BlockDev& Bk = tab[blockIdx.y];
  // (scheme-9 blocks only: a scheme-1 block assembled in FP32 is solved
  // in FP64 by vic_solve3_kernel)
  if (Bk.implicit != 9 || !Bk.implicit_f32) return;
  const VicScratch S = vic_scratch(Bk);
  const int n = Bk.nc1 - 2 * Bk.ng;
  const VicScratch32 F = vic_scratch32(Bk, S, n);
  const size_t ncol = F.ncol;
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  const size_t warp = (size_t)blockIdx.x * kCorrWarps + wl;
  if (warp * kCorrCols >= ncol) return;  // the whole warp
  CorrSlot* sl = ring[wl];
  const int cl = lane / 3, k = lane - 3 * cl;
  const int base = 3 * cl;  // the column's first lane
  const size_t col = warp * kCorrCols + cl;
  const bool wood = n >= 3;
  // a lane past the warp's columns shadows the warp's first column; it
  // neither copies nor stores
  const bool valid = cl < kCorrCols && col < ncol;
  const size_t cc = valid ? col : warp * kCorrCols;
  const bool live = valid && F.mask[cc] == 0;
  const bool act = live && (k == 0 || wood);
  const int cs = cl < kCorrCols ? cl : 0;  // the lane's column slot
  const unsigned full = 0xffffffffu;
  // true on every lane of this lane's column (inactive lanes agree)
  auto all3 = [&](bool v) {
    const unsigned bad = __ballot_sync(full, !v);
    return ((bad >> base) & 7u) == 0u;
  };
  const float* LU = F.LU + cc * n * kLu32;
  const float* Bm = F.B + cc * n * kBlk32;
  const float* CP = F.CP + cc * n * kBlk32;
  float* R = F.R + cc * n * kR32;
  double* X = (k == 0 ? S.D : (k == 1 ? S.Z0 : S.Z1)) + cc * n * 5;

  // ---- forward: y_i = LU_i^-1 (r_i - b_i y_(i-1)) ----
  // the column's three lanes share the copies of its layer
  auto fissue = [&](int i) {
    if (live) {
      CorrSlot& s = sl[i % kCorrRing];
      for (int e = k; e < kLu32 / 4; e += 3)
        cpa16(&s.f.lu[cs][4 * e], LU + i * kLu32 + 4 * e);
      for (int e = k; e < kBlk32 / 4; e += 3)
        cpa16(&s.f.b[cs][4 * e], Bm + i * kBlk32 + 4 * e);
      for (int e = k; e < kR32 / 4; e += 3)
        cpa16(&s.f.r[cs][4 * e], R + i * kR32 + 4 * e);
    }
  };
#pragma unroll
  for (int j = 0; j < kCorrRing - 1; ++j) {
    if (j < n) fissue(j);
    cpa_commit();
  }
  float y[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  for (int i = 0; i < n; ++i) {
    if (i + kCorrRing - 1 < n) fissue(i + kCorrRing - 1);
    cpa_commit();
    cpa_wait<kCorrRing - 1>();
    __syncwarp();
    const CorrSlot& s = sl[i % kCorrRing];
    if (act) {
      const float* lu = s.f.lu[cs];
      const float* b = s.f.b[cs];
      float x[5];
#pragma unroll
      for (int r = 0; r < 5; ++r) x[r] = s.f.r[cs][k * 5 + r];
      if (i > 0) {
#pragma unroll
        for (int r = 0; r < 5; ++r) {
          float t = x[r];
#pragma unroll
          for (int q = 0; q < 5; ++q) t = fmaf(-b[r * 5 + q], y[q], t);
          x[r] = t;
        }
      }
      const int pk = __float_as_int(lu[30]);
#pragma unroll
      for (int rr = 0; rr < 5; ++rr) {
        const int ip = (pk >> (3 * rr)) & 7;
#pragma unroll
        for (int q = rr + 1; q < 5; ++q) {
          const bool sw = ip == q;
          const float a = x[rr], c = x[q];
          x[rr] = sw ? c : a;
          x[q] = sw ? a : c;
        }
      }
#pragma unroll
      for (int rr = 1; rr < 5; ++rr)
#pragma unroll
        for (int jj = 0; jj < rr; ++jj)
          x[rr] = fmaf(-lu[rr * 5 + jj], x[jj], x[rr]);
#pragma unroll
      for (int rr = 4; rr >= 0; --rr) {
#pragma unroll
        for (int jj = rr + 1; jj < 5; ++jj)
          x[rr] = fmaf(-lu[rr * 5 + jj], x[jj], x[rr]);
        x[rr] = x[rr] * lu[25 + rr];
      }
#pragma unroll
      for (int r = 0; r < 5; ++r) {
        R[i * kR32 + k * 5 + r] = x[r];  // y, for the way back
        y[r] = x[r];
      }
    }
    __syncwarp();  // the slot is read before it is refilled
  }
  cpa_wait<0>();
  __syncwarp();

  // ---- back: d_i = y_i - c'_i d_(i+1), x_i += d_i in FP64 ----
  float dmax = 0.f;
  bool fin = true;
  // a correction before the last keeps d for the next residual (r - T d),
  // in the C scratch (unused by the refined solve otherwise)
  float* DD = reinterpret_cast<float*>(S.C) + cc * n * kR32 + k * 5;
  if (act) {
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      if (!last) DD[(n - 1) * kR32 + r] = y[r];
      X[(n - 1) * 5 + r] = X[(n - 1) * 5 + r] + widen_exact(y[r]);
      fin = fin && vfinite32(y[r]);
      dmax = fmaxf(dmax, fabsf(y[r]));
    }
  }
  // step j of the way back is layer n - 2 - j
  auto bissue = [&](int j) {
    const int i = n - 2 - j;
    CorrSlot& s = sl[j % kCorrRing];
    if (live) {
      for (int e = k; e < kBlk32 / 4; e += 3)
        cpa16(&s.g.cp[cs][4 * e], CP + i * kBlk32 + 4 * e);
      for (int e = k; e < kR32 / 4; e += 3)
        cpa16(&s.g.y[cs][4 * e], R + i * kR32 + 4 * e);
    }
    if (act) {
#pragma unroll
      for (int r = 0; r < 5; ++r) cpa8(&s.g.x[lane][r], X + i * 5 + r);
    }
  };
#pragma unroll
  for (int j = 0; j < kCorrRing - 1; ++j) {
    if (j < n - 1) bissue(j);
    cpa_commit();
  }
  for (int j = 0; j < n - 1; ++j) {
    const int i = n - 2 - j;
    if (j + kCorrRing - 1 < n - 1) bissue(j + kCorrRing - 1);
    cpa_commit();
    cpa_wait<kCorrRing - 1>();
    __syncwarp();
    const CorrSlot& s = sl[j % kCorrRing];
    if (act) {
      const float* cp = s.g.cp[cs];
      float t[5];
#pragma unroll
      for (int r = 0; r < 5; ++r) {
        float u = s.g.y[cs][k * 5 + r];
#pragma unroll
        for (int q = 0; q < 5; ++q) u = fmaf(-cp[r * 5 + q], y[q], u);
        t[r] = u;
      }
#pragma unroll
      for (int r = 0; r < 5; ++r) {
        y[r] = t[r];
        if (!last) DD[i * kR32 + r] = t[r];
        X[i * 5 + r] = s.g.x[lane][r] + widen_exact(t[r]);
        fin = fin && vfinite32(t[r]);
        dmax = fmaxf(dmax, fabsf(t[r]));
      }
    }
    __syncwarp();
  }
  cpa_wait<0>();

  float* st = F.stat + cc * 6;
  if (!last) {
    const bool colok = all3(!act || fin);
    if (act) st[k] = dmax;
    if (live && k == 0 && !colok) F.mask[cc] = 1;
    return;
  }
  // convergence of every right-hand side of the column
  bool cv = true;
  if (act) {
    const float dp = st[k];
    const float rho = dp > 0.f ? fminf(dmax / dp, 1.f) : 0.f;
    cv = fin && dmax * rho <= 0x1p-44f * st[3 + k];
    st[k] = dmax;  // the last update, kept for inspection (nothing reads it)
  }
  // every ballot runs on all 32 lanes: evaluate before combining
  const bool cv_all = all3(cv);
  bool conv = live && cv_all;
  // the Woodbury step of each converged column: its first lane forms the
  // two weights from D, Z0, Z1 at layers 2 and n - 3, then the whole warp
  // updates the column's 5 n values of D, coalesced, one column at a time
  __syncwarp();  // every lane's x is stored
  double al0 = 0., al1 = 0.;
  if (conv && wood && k == 0) {
    const double* D = S.D + cc * n * 5;
    const double* Z0 = S.Z0 + cc * n * 5;
    const double* Z1 = S.Z1 + cc * n * 5;
    const double dtc = p.w2 * p.dt[blockIdx.y];
    VicK K0 = vic_krows(Bk, n, 0), K1 = vic_krows(Bk, n, n - 1);
    const double k0 = -K0.t0 / dtc, k1 = -K1.t1 / dtc;
    const int a0 = 2, a1 = n - 3;
    const double m00 = 1. + k0 * Z0[a0 * 5], m01 = k0 * Z1[a0 * 5];
    const double m10 = k1 * Z0[a1 * 5], m11 = 1. + k1 * Z1[a1 * 5];
    const double r0 = k0 * D[a0 * 5], r1 = k1 * D[a1 * 5];
    const double det = m00 * m11 - m01 * m10;
    al0 = (m11 * r0 - m01 * r1) / det;
    al1 = (m00 * r1 - m10 * r0) / det;
  }
  const unsigned wb = __ballot_sync(full, conv && wood && k == 0);
  __syncwarp();  // the weights are read before D changes
  bool bad = false;  // on a column's first lane: its D is not finite
  for (int c = 0; c < kCorrCols; ++c) {
    if (!((wb >> (3 * c)) & 1u)) continue;  // uniform over the warp
    const double w0 = __shfl_sync(full, al0, 3 * c);
    const double w1 = __shfl_sync(full, al1, 3 * c);
    const size_t cw = warp * kCorrCols + c;
    double* D = S.D + cw * n * 5;
    const double* Z0 = S.Z0 + cw * n * 5;
    const double* Z1 = S.Z1 + cw * n * 5;
    bool f = true;
    for (int e = lane; e < 5 * n; e += 32) {
      double d = D[e];
      d -= Z0[e] * w0;
      d -= Z1[e] * w1;
      D[e] = d;
      f = f && vfinite(d);
    }
    const bool f_all = __all_sync(full, f);
    if (lane == 3 * c) bad = !f_all;
  }
  if (valid && k == 0) F.mask[cc] = (conv && !bad) ? 0 : 1;
}

// implicit-solve fp32 (the reference's FP32 compute of the implicit solve,
// the PrecisionPolicy's kImplicit row in FP32): after the FP32 sweep, the
// Woodbury step of every column the sweep solved, in FP64 on its widened
// FP32 solution, one warp per column (coalesced over the 5 n values); a
// column whose sweep failed, or whose result is not finite, stays masked for
// the direct FP64 solve (the reference's FP64 retry of the failed columns)
__global__ void __launch_bounds__(kThreads)
    vic_woodbury32_kernel(const BlockDev* __restrict__ tab, StageParams p) {
  const BlockDev& Bk = tab[blockIdx.y];
  // (scheme-9 blocks only: a scheme-1 block assembled in FP32 is solved
  // in FP64 by vic_solve3_kernel)
  if (Bk.implicit != 9 || !Bk.implicit_f32) return;
  const VicScratch S = vic_scratch(Bk);
  const int n = Bk.nc1 - 2 * Bk.ng;
  const VicScratch32 F = vic_scratch32(Bk, S, n);
  const size_t col = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (col >= F.ncol || F.mask[col]) return;  // uniform over the warp
  double* D = S.D + col * n * 5;
  const double* Z0 = S.Z0 + col * n * 5;
  const double* Z1 = S.Z1 + col * n * 5;
  if (n < 3) return;  // no Woodbury step; the sweep screened the solution
  const double dtc = p.w2 * p.dt[blockIdx.y];
  VicK K0 = vic_krows(Bk, n, 0), K1 = vic_krows(Bk, n, n - 1);
  const double k0 = -K0.t0 / dtc, k1 = -K1.t1 / dtc;
  const int a0 = 2, a1 = n - 3;
  const double m00 = 1. + k0 * Z0[a0 * 5], m01 = k0 * Z1[a0 * 5];
  const double m10 = k1 * Z0[a1 * 5], m11 = 1. + k1 * Z1[a1 * 5];
  const double r0 = k0 * D[a0 * 5], r1 = k1 * D[a1 * 5];
  const double det = m00 * m11 - m01 * m10;
  const double al0 = (m11 * r0 - m01 * r1) / det;
  const double al1 = (m00 * r1 - m10 * r0) / det;
  __syncwarp();  // every lane has read the weights' inputs
  bool f = true;
  for (int e = lane; e < 5 * n; e += 32) {
    double d = D[e];
    d -= Z0[e] * al0;
    d -= Z1[e] * al1;
    D[e] = d;
    f = f && vfinite(d);
  }
  if (!__all_sync(0xffffffffu, f) && lane == 0) F.mask[col] = 1;
}

// s_h + s_l += t d in float-float arithmetic, t and d floats: the product
// split exactly by an FMA (the two-product of Dekker's method), the sum by
// Knuth's two-sum; the low parts gather in s_l.  Every step is a single
// rounding (__fmul_rn / __fadd_rn are never contracted)
__device__ __forceinline__ void ff_madd(float& sh, float& sl, float t, float d) {
  const float p = __fmul_rn(t, d);
  const float e = __fmaf_rn(t, d, -p);
  const float s2 = __fadd_rn(sh, p);
  const float bp = __fadd_rn(s2, -sh);
  const float err =
      __fadd_rn(__fadd_rn(sh, -__fadd_rn(s2, -bp)), __fadd_rn(p, -bp));
  sl = __fadd_rn(sl, __fadd_rn(err, e));
  sh = s2;
}

// s_h + (m_h + m_l) += t d, t and d floats, to well beyond FP64 accuracy:
// the product split exactly (Dekker's two-product by an FMA), its high part
// added to s_h by Knuth's two-sum, and the two exact remainders (the sum's
// rounding error and the product's low part) gathered in the float-float
// pair m_h + m_l.  The pair holds terms of 2^-24 of the products, so its
// own error is about 2^-48 of that: 2^-72 of the sum of |t d|
__device__ __forceinline__ void ff_acc(float& mh, float& ml, float v) {
  const float s2 = __fadd_rn(mh, v);
  const float bp = __fadd_rn(s2, -mh);
  ml = __fadd_rn(ml, __fadd_rn(__fadd_rn(mh, -__fadd_rn(s2, -bp)),
                               __fadd_rn(v, -bp)));
  mh = s2;
}

__device__ __forceinline__ void tf_madd(float& sh, float& mh, float& ml, float t,
                                        float d) {
  const float p = __fmul_rn(t, d);
  const float e = __fmaf_rn(t, d, -p);
  const float s2 = __fadd_rn(sh, p);
  const float bp = __fadd_rn(s2, -sh);
  const float err =
      __fadd_rn(__fadd_rn(sh, -__fadd_rn(s2, -bp)), __fadd_rn(p, -bp));
  sh = s2;
  ff_acc(mh, ml, err);
  ff_acc(mh, ml, e);
}

// the residual r = b - (B_i x_(i-1) + A_i x_i + C_i x_(i+1)) of every cell
// and right-hand side (one thread per cell), rounded to FP32 into R for the
// correction's sweeps.
// * The first correction (corr 1) forms it from the FP32-assembled blocks
//   and x in D, Z0, Z1, which the FP32 sweep wrote as floats widened
//   (exact): T x as a sum of exact float products (tf_madd, on the FP32
//   pipe, to about 2^-72 of the sum of |t x|), then b minus that sum in
//   FP64 (three subtractions, the first exact); it keeps the FP64 r (in the
//   B scratch, which the refined solve does not use otherwise).  Formed
//   with FP64 multiply-adds instead, the sum took 225 FP64 instructions per
//   cell and kept the FP64 pipe 83 % busy; its rounding, 2^-53 per add,
//   was the coarser of the two.
// * A later correction forms it from the previous one: x grew by the FP32
//   correction d (kept in the C scratch by vic_correct32_kernel), so
//   r_new = r - T d.  T and d are floats, so T d is summed in float-float
//   on the FP32 pipe (its error, 2^-48 of the sum of |t d| with |d| about
//   2^-20 |x|, is far below the FP64 rounding of r); the two FP64 subtractions
//   that remain replace 225 FP64 multiply-adds per cell.  The rounding of
//   x += d in FP64 adds at most 2^-53 |x| to x, the FP64 residual's own level.
#ifndef SG_RES_THREADS
#define SG_RES_THREADS 256
#endif
constexpr int kResThreads = SG_RES_THREADS;
__global__ void __launch_bounds__(kResThreads)
    vic_residual_kernel(const BlockDev* __restrict__ tab, StageParams p,
                        int corr) {
  const BlockDev& B = tab[blockIdx.y];
  if (B.implicit != 9 || !B.implicit_f32) return;  // scheme 9 only
  const VicScratch S = vic_scratch(B);
  const int n = B.nc1 - 2 * B.ng;
  const VicScratch32 F = vic_scratch32(B, S, n);
  const double dtc = p.w2 * p.dt[blockIdx.y];
  const double rdtc = 1. / dtc;
  const int nrhs = n >= 3 ? 3 : 1;
  const bool keep = corr < p.refine;  // a later correction reads r
  const float* DD = reinterpret_cast<const float*>(S.C);
  for (size_t cell = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
       cell < S.cells; cell += (size_t)gridDim.x * blockDim.x) {
    const size_t col = cell / n;
    const int i = (int)(cell - col * n);
    if (F.mask[col]) continue;
    const float* a = F.A + cell * kBlk32;
    const float* bl = F.B + cell * kBlk32;
    const float* c = F.C + cell * kBlk32;
    for (int k = 0; k < nrhs; ++k) {
      double* rb = S.B + cell * 25 + k * 5;
      double t[5];
      if (corr == 1) {
        const double* x = (k == 0 ? S.D : (k == 1 ? S.Z0 : S.Z1)) + cell * 5;
        float sh[5] = {0.f, 0.f, 0.f, 0.f, 0.f}, mh[5] = {0.f, 0.f, 0.f, 0.f, 0.f},
              ml[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int q = 0; q < 5; ++q) {
          const float xc = narrow_exact(x[q]);
#pragma unroll
          for (int r = 0; r < 5; ++r) tf_madd(sh[r], mh[r], ml[r], a[r * 5 + q], xc);
        }
        if (i > 0) {
#pragma unroll
          for (int q = 0; q < 5; ++q) {
            const float xl = narrow_exact(x[q - 5]);
#pragma unroll
            for (int r = 0; r < 5; ++r) tf_madd(sh[r], mh[r], ml[r], bl[r * 5 + q], xl);
          }
        }
        if (i < n - 1) {
#pragma unroll
          for (int q = 0; q < 5; ++q) {
            const float xu = narrow_exact(x[q + 5]);
#pragma unroll
            for (int r = 0; r < 5; ++r) tf_madd(sh[r], mh[r], ml[r], c[r * 5 + q], xu);
          }
        }
#pragma unroll
        for (int r = 0; r < 5; ++r) {
          const double b = k == 0 ? vdiv(S.du[(size_t)r * S.cells + cell], dtc, rdtc)
                                  : ((r == 4 && i == (k == 1 ? 0 : n - 1)) ? 1. : 0.);
          t[r] = ((b - widen_exact(sh[r])) - widen_exact(mh[r])) - widen_exact(ml[r]);
        }
      } else {
        float sh[5] = {0.f, 0.f, 0.f, 0.f, 0.f}, sl[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
        const float* dc = DD + cell * kR32 + k * 5;
#pragma unroll
        for (int q = 0; q < 5; ++q) {
          const float dq = dc[q];
#pragma unroll
          for (int r = 0; r < 5; ++r) ff_madd(sh[r], sl[r], a[r * 5 + q], dq);
        }
        if (i > 0) {
#pragma unroll
          for (int q = 0; q < 5; ++q) {
            const float dq = dc[q - kR32];
#pragma unroll
            for (int r = 0; r < 5; ++r) ff_madd(sh[r], sl[r], bl[r * 5 + q], dq);
          }
        }
        if (i < n - 1) {
#pragma unroll
          for (int q = 0; q < 5; ++q) {
            const float dq = dc[q + kR32];
#pragma unroll
            for (int r = 0; r < 5; ++r) ff_madd(sh[r], sl[r], c[r * 5 + q], dq);
          }
        }
#pragma unroll
        for (int r = 0; r < 5; ++r)
          t[r] = (rb[r] - widen_exact(sh[r])) - widen_exact(sl[r]);
      }
#pragma unroll
      for (int r = 0; r < 5; ++r) {
        if (keep) rb[r] = t[r];
        F.R[cell * kR32 + k * 5 + r] = narrow_exact(t[r]);
      }
    }
  }
}

// NL lanes per column: 32 (a warp per column, kVicWarps per CTA: the serial
// passes on lane 0, the per-layer maps on every lane) or 1 (a thread per
// column, for batches with enough columns to fill the GPU: every FP64
// instruction of the serial passes then serves 32 columns).  The operations
// and their order are the same in both.
template <int NL>
__global__ void __launch_bounds__(NL == 32 ? 32 * kVicWarps : kThreads)
    vic_finish_kernel(const BlockDev* __restrict__ tab, StageParams p) {
  const BlockDev& B = tab[blockIdx.y];
  if (!B.implicit) return;
  const int lane = NL == 32 ? (threadIdx.x & 31) : 0;
  const VicScratch S = vic_scratch(B);
  const int ng = B.ng, nc1 = B.nc1, n = nc1 - 2 * ng;
  const size_t ncol = S.cells / n;
  const size_t col = NL == 32 ? (size_t)blockIdx.x * kVicWarps + (threadIdx.x >> 5)
                              : (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;  // whole warps leave together when NL = 32
  const size_t plane = (size_t)nc1 * B.nc2 * B.nc3;
  const real* uin = static_cast<const real*>(B.buf[p.in]);
  const real* u0 = static_cast<const real*>(B.buf[p.u0]);
  real* uout = static_cast<real*>(B.buf[p.out]);
  const size_t jrow = vic_row(B, col);
  const size_t base = jrow * nc1 + ng;
  const double grav = B.grav1;
  const double vol = B.dx3 * (B.dx2 * B.dx1);
  const double rvol = 1. / vol;  // the quotients by vol divide by it (vdiv)
  const double* x1v = B.x1v + ng;
  const double* x1f = B.x1f + ng;
  const double* D = S.D + col * n * 5;
  double* du = S.du + col * n;      // row v at du[v * cells + i]
  const double* du0 = S.du0 + col * n;
  const size_t cs = S.cells;
  const bool ok = vfinite(D[0]);
  const bool wood = n >= 3;
  // work arrays of the column, in the (now free) Woodbury scratch
  // the warp form keeps a column's arrays contiguous; the thread form
  // interleaves the columns (index i at i ncol + col), so a warp's 32
  // columns read and write consecutive doubles
  const size_t ws = NL == 32 ? 1 : ncol;
  double* const w0p = NL == 32 ? S.Z0 + col * n * 5 : S.Z0 + col;
  const VCol mM{w0p, ws};                                  // n + 1: the face mass below layer i
  const VCol mq{w0p + (size_t)(n + 1) * ws, ws};           // n + 1: the moved total mass
  const VCol mdn{w0p + (size_t)(2 * n + 2) * ws, ws};      // n: the dry-gas increment
  const VCol rho{w0p + (size_t)(3 * n + 2) * ws, ws};      // n: the density of each layer
  // the partial matrix (implicit-scheme 1): the tangential velocities of
  // layers 0..n (n: the ghost above), in the (free) second Woodbury vector
  const bool partial = B.implicit == 1;
  double* const w1p = NL == 32 ? S.Z1 + col * n * 5 : S.Z1 + col;
  const VCol vt2{w1p, ws}, vt3{w1p + (size_t)(n + 1) * ws, ws};
  if (ok) {
    for (int i = lane; i < n; i += NL) {
      double w[5];
      vic_prim(uin, plane, base + i, B.gammad, w, B.base, nc1);
      rho[i] = w[0];
      mdn[i] = 0.;
      mq[i] = (D[i * 5] - du[i]) * vol;  // staged: phi of layer i
      if (partial) {
        vt2[i] = w[2];
        vt3[i] = w[3];
      }
    }
    if (partial && lane == 0) {
      double w[5];
      vic_prim(uin, plane, base + n, B.gammad, w, B.base, nc1);
      vt2[n] = w[2];
      vt3[n] = w[3];
    }
    vsync<NL>();
    if (lane == 0) {
      double R = 0, Ssum = 0;
      for (int i = 0; i < n; ++i) {
        R += mq[i];
        Ssum += rho[i] * vol;
      }
      double M = 0;
      const double rss = 1. / Ssum;
      for (int i = 0; i < n; ++i) {
        mM[i] = M;
        M -= mq[i] - R * vdiv(rho[i] * vol, Ssum, rss);
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
        const double qv = vdiv(q, vol, rvol);
        mdn[i] -= qv;
        mdn[i + 1] += qv;
        mq[i + 1] = q;
        avail = avail_up + q;
      }
    }
    vsync<NL>();
    for (int i = lane; i < n; i += NL) {
      du[i] += mdn[i];
      du[cs + i] = D[i * 5 + 1];
      if (!partial) {  // the partial matrix keeps the explicit m_t rows
        du[2 * cs + i] = D[i * 5 + 2];
        du[3 * cs + i] = D[i * 5 + 3];
      }
      double e = D[i * 5 + 4];
      double projected = vdiv(mM[i] - mM[i + 1], vol, rvol);
      double ph = -grav * x1v[i];
      double pw = ph * (D[i * 5] - du0[i] - projected);
      double dp_lo = -grav * (x1f[i] - x1v[i]);
      double dp_hi = -grav * (x1f[i + 1] - x1v[i]);
      double mv_lo = mq[i] - mM[i], mv_hi = mq[i + 1] - mM[i + 1];
      double cw = vdiv(-(dp_hi * mv_hi - dp_lo * mv_lo), vol, rvol);
      du[4 * cs + i] = e + (pw + cw);
    }
    vsync<NL>();
    if (partial && lane == 0) {
      // vic_tangential_momentum_column (src/implicit/vic_redistribute_impl.h
      // :178-200): each face's moved total mass carries the donor (upwind)
      // cell's tangential velocity; a zero transfer leaves du as it is
      for (int i = 0; i + 1 < n; ++i) {
        const double q = mq[i + 1];
        const int donor = q > 0 ? i : i + 1;
        const double pm[2] = {q * vt2[donor], q * vt3[donor]};
#pragma unroll
        for (int t = 0; t < 2; ++t) {
          if (pm[t] == 0) continue;
          du[(2 + t) * cs + i] -= vdiv(pm[t], vol, rvol);
          du[(2 + t) * cs + i + 1] += vdiv(pm[t], vol, rvol);
        }
      }
    }
    vsync<NL>();
    if (wood) {
      // the remainder g1 sigma^2 s[du - du0] - K (raw - du0) of each layer,
      // from the final IDN row of its neighbours
      // staged in mdn (free again): every layer's work reads the IDN row
      // only, so the IPR row is written after all of them
      for (int i = lane; i < n; i += NL) {
        double wt[3];
        int i0;
        vic_slope_tab(B, n, i, wt, &i0);
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
      vsync<NL>();
      for (int i = lane; i < n; i += NL) du[4 * cs + i] += mdn[i];
    }
    vsync<NL>();
  }
  // passive scalars: the clamped dry transfer of each x1 face (zero for a
  // failed column), for their share of it
  if (B.nscalar > 0)
    for (int f = lane; f <= n; f += NL)
      B.vicq[jrow * nc1 + ng + f] = ok ? (double)mq[f] : 0.;
  // the x1 step field of an implicit block (FluxRegister::end_stage after
  // ImplicitHydroImpl::post_, src/implicit/implicit_hydro.cpp:625-673): the
  // stage's T_1 plus the solve's face transfers per unit area and time,
  // "vic.mass_dry" q / (dt A) on row IDN and "vic.momentum_t"
  // -sum_{k < f} (du - du0)_k V / (dt A) on rows IVY and IVZ (the prefix from
  // the bottom wall, top face included), then the prescribed wall faces.  A
  // failed column posts nothing.  Each face's adds run in the reference's
  // order, +0 posts included (a -0 total becomes +0)
  if (double* S1 = B.step[0]) {
    const double dt = p.dt[blockIdx.y];
    const double kdt = dt * (B.dx3 * B.dx2), rkdt = 1. / kdt;
    const double w1s = p.w1, w2dt = p.w2 * dt;
    const bool first = p.first != 0;
    const int nf = n + 1;
    const double* T = B.t1;
    const bool wlo = B.bc[0] == kBcReflecting, whi = B.bc[1] == kBcReflecting;
    auto tot = [&](int v, int f) { return T[((size_t)v * ncol + col) * nf + f]; };
    auto at = [&](int v, int f) { return S1 + v * plane + jrow * nc1 + ng + f; };
    for (int f = lane; f < nf; f += NL) {
      double t0 = tot(IDN, f), t1 = tot(IVX, f), t4 = tot(IPR, f);
      if (ok) t0 = t0 + vdiv(mq[f], kdt, rkdt);
      if ((f == 0 && wlo) || (f == n && whi)) t0 = t4 = 0.;
      step_set(at(IDN, f), t0, w1s, w2dt, first);
      step_set(at(IVX, f), t1, w1s, w2dt, first);
      step_set(at(IPR, f), t4, w1s, w2dt, first);
    }
    if (lane == 0) {
      double sy = 0., sz = 0.;
      for (int f = 0; f < nf; ++f) {
        double ty = tot(IVY, f), tz = tot(IVZ, f);
        if (ok && partial) {
          // the partial matrix posts the donor transfer q w_t of each face
          // (src/implicit/implicit_hydro.cpp:520-530,662-666)
          const double q = mq[f];
          const int donor = q > 0. ? f - 1 : f;
          ty = ty + vdiv(q * vt2[donor], kdt, rkdt);
          tz = tz + vdiv(q * vt3[donor], kdt, rkdt);
        } else if (ok) {
          double py = 0., pz = 0.;
          if (f > 0) {
            sy = sy + (D[(f - 1) * 5 + 2] - du0[2 * cs + f - 1]) * vol;
            sz = sz + (D[(f - 1) * 5 + 3] - du0[3 * cs + f - 1]) * vol;
            py = -sy;
            pz = -sz;
          }
          ty = ty + vdiv(py, kdt, rkdt);
          tz = tz + vdiv(pz, kdt, rkdt);
        }
        step_set(at(IVY, f), ty, w1s, w2dt, first);
        step_set(at(IVZ, f), tz, w1s, w2dt, first);
      }
    }
  }
  // the RK combine of the column (a failed column keeps the explicit du)
  const double* dsel = ok ? S.du + col * n : du0;
  const real w0 = real(p.w0), w1 = real(p.w1), w2 = real(p.w2);
  for (int i = lane; i < n; i += NL) {
    const size_t c = base + i;
#pragma unroll
    for (int v = 0; v < NHYDRO; ++v) {
      const size_t q = v * plane + c;
      uout[q] = w0 * u0[q] + w1 * uin[q] + w2 * real(dsel[v * cs + i]);
    }
  }
}

// ---------------------------------------------------------------------------
// (3w) the finish of wide batches in three launches.  A thread per column
// walks every layer serially and, with a few warps per SM, waits on memory
// at each one; here only the constituent column's serial scans keep a
// thread per column, and the per-layer work runs a thread per cell:
//   vic_finish_a_kernel  per cell: the layer's density (and, for the partial
//                        matrix, its tangential velocities) and phi =
//                        (D_rho - du_rho) V
//   vic_finish_b_kernel  per column: the sums R and S, the face-mass prefix
//                        M, the availability clamp (q, the dry increment),
//                        the scalars' face transfers and the x1 step field
//   vic_finish_c_kernel  per cell: the map of the solution, the partial
//                        matrix's tangential transfers, the gravity-work
//                        remainder and the RK combine, from the inputs only
//                        (no cell writes what another reads)
// Every value takes the operations of vic_finish_kernel in its order, so
// the results are the same bit for bit.  A column's work arrays stay in its
// (free) Woodbury scratch, column-contiguous:
//   Z0: mM [n + 1] | mq [n + 1] | mdn [n] | rho [n]
//   Z1: vt2 [n + 1] | vt3 [n + 1] | phi [n]
struct FinishCol {
  double *mM, *mq, *mdn, *rho, *vt2, *vt3, *phi;
};

__device__ __forceinline__ FinishCol finish_col(const VicScratch& S,
                                                size_t col, int n) {
  double* z0 = S.Z0 + col * n * 5;
  double* z1 = S.Z1 + col * n * 5;
  return FinishCol{z0, z0 + (n + 1), z0 + (2 * n + 2), z0 + (3 * n + 2),
                   z1, z1 + (n + 1), z1 + (2 * n + 2)};
}

__global__ void __launch_bounds__(kThreads)
    vic_finish_a_kernel(const BlockDev* __restrict__ tab, StageParams p) {
  const BlockDev& B = tab[blockIdx.y];
  if (!B.implicit) return;
  const VicScratch S = vic_scratch(B);
  const int ng = B.ng, nc1 = B.nc1, n = nc1 - 2 * ng;
  const size_t plane = (size_t)nc1 * B.nc2 * B.nc3;
  const real* uin = static_cast<const real*>(B.buf[p.in]);
  const double vol = B.dx3 * (B.dx2 * B.dx1);
  const bool partial = B.implicit == 1;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < S.cells;
       e += (size_t)gridDim.x * blockDim.x) {
    const size_t col = e / n;
    const int i = (int)(e - col * n);
    const double* D = S.D + col * n * 5;
    if (!vfinite(D[0])) continue;
    const size_t base = vic_row(B, col) * nc1 + ng;
    const FinishCol F = finish_col(S, col, n);
    double w[5];
    vic_prim(uin, plane, base + i, B.gammad, w, B.base, nc1);
    F.rho[i] = w[0];
    F.phi[i] = (D[i * 5] - S.du[e]) * vol;
    if (partial) {
      F.vt2[i] = w[2];
      F.vt3[i] = w[3];
      if (i == n - 1) {  // the ghost above, the donor of the top face
        vic_prim(uin, plane, base + n, B.gammad, w, B.base, nc1);
        F.vt2[n] = w[2];
        F.vt3[n] = w[3];
      }
    }
  }
}

// a thread per column: small CTAs spread a batch's few columns (21,120 for
// the 64-member ensemble) over every SM (one box, the ensemble's finish:
// 514 us per stage with 256 threads, 472 with 64, 463 with 32)
#ifndef SG_FINISH_B_THREADS
#define SG_FINISH_B_THREADS 32
#endif
constexpr int kFinishBThreads = SG_FINISH_B_THREADS;
__global__ void __launch_bounds__(kFinishBThreads)
    vic_finish_b_kernel(const BlockDev* __restrict__ tab, StageParams p) {
  const BlockDev& B = tab[blockIdx.y];
  if (!B.implicit) return;
  const VicScratch S = vic_scratch(B);
  const int ng = B.ng, nc1 = B.nc1, n = nc1 - 2 * ng;
  const size_t ncol = S.cells / n;
  const size_t col = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const size_t plane = (size_t)nc1 * B.nc2 * B.nc3;
  const size_t jrow = vic_row(B, col);
  const double vol = B.dx3 * (B.dx2 * B.dx1);
  const double rvol = 1. / vol;
  const double* D = S.D + col * n * 5;
  const double* du = S.du + col * n;
  const double* du0 = S.du0 + col * n;
  const size_t cs = S.cells;
  const bool ok = vfinite(D[0]);
  const bool partial = B.implicit == 1;
  const FinishCol F = finish_col(S, col, n);
  if (ok) {
    double R = 0, Ssum = 0;
    for (int i = 0; i < n; ++i) {
      R += F.phi[i];
      Ssum += F.rho[i] * vol;
    }
    double M = 0;
    const double rss = 1. / Ssum;
    for (int i = 0; i < n; ++i) {
      F.mM[i] = M;
      M -= F.phi[i] - R * vdiv(F.rho[i] * vol, Ssum, rss);
    }
    F.mM[n] = 0.;
    F.mq[0] = 0.;
    double avail = (F.rho[0] * 1. + du[0]) * vol;
    if (avail < 0) avail = 0;
    double dn = 0.;  // the dry increment of layer i, carried up
    for (int i = 0; i + 1 < n; ++i) {
      double avail_up = (F.rho[i + 1] * 1. + du[i + 1]) * vol;
      if (avail_up < 0) avail_up = 0;
      double Mf = F.mM[i + 1];
      double q = Mf > 0 ? Mf * 1. : Mf * 1.;
      if (q > avail) q = avail;
      if (q < -avail_up) q = -avail_up;
      const double qv = vdiv(q, vol, rvol);
      F.mdn[i] = dn - qv;
      dn = 0. + qv;
      F.mq[i + 1] = q;
      avail = avail_up + q;
    }
    F.mdn[n - 1] = dn;
    F.mq[n] = 0.;
  }
  if (B.nscalar > 0)
    for (int f = 0; f <= n; ++f)
      B.vicq[jrow * nc1 + ng + f] = ok ? F.mq[f] : 0.;
  // the x1 step field, as in vic_finish_kernel
  if (double* S1 = B.step[0]) {
    const double dt = p.dt[blockIdx.y];
    const double kdt = dt * (B.dx3 * B.dx2), rkdt = 1. / kdt;
    const double w1s = p.w1, w2dt = p.w2 * dt;
    const bool first = p.first != 0;
    const int nf = n + 1;
    const double* T = B.t1;
    const bool wlo = B.bc[0] == kBcReflecting, whi = B.bc[1] == kBcReflecting;
    auto tot = [&](int v, int f) { return T[((size_t)v * ncol + col) * nf + f]; };
    auto at = [&](int v, int f) { return S1 + v * plane + jrow * nc1 + ng + f; };
    double sy = 0., sz = 0.;
    for (int f = 0; f < nf; ++f) {
      double t0 = tot(IDN, f), t1 = tot(IVX, f), t4 = tot(IPR, f);
      if (ok) t0 = t0 + vdiv(F.mq[f], kdt, rkdt);
      if ((f == 0 && wlo) || (f == n && whi)) t0 = t4 = 0.;
      step_set(at(IDN, f), t0, w1s, w2dt, first);
      step_set(at(IVX, f), t1, w1s, w2dt, first);
      step_set(at(IPR, f), t4, w1s, w2dt, first);
      double ty = tot(IVY, f), tz = tot(IVZ, f);
      if (ok && partial) {
        const double q = F.mq[f];
        const int donor = q > 0. ? f - 1 : f;
        ty = ty + vdiv(q * F.vt2[donor], kdt, rkdt);
        tz = tz + vdiv(q * F.vt3[donor], kdt, rkdt);
      } else if (ok) {
        double py = 0., pz = 0.;
        if (f > 0) {
          sy = sy + (D[(f - 1) * 5 + 2] - du0[2 * cs + f - 1]) * vol;
          sz = sz + (D[(f - 1) * 5 + 3] - du0[3 * cs + f - 1]) * vol;
          py = -sy;
          pz = -sz;
        }
        ty = ty + vdiv(py, kdt, rkdt);
        tz = tz + vdiv(pz, kdt, rkdt);
      }
      step_set(at(IVY, f), ty, w1s, w2dt, first);
      step_set(at(IVZ, f), tz, w1s, w2dt, first);
    }
  }
}

__global__ void __launch_bounds__(kThreads)
    vic_finish_c_kernel(const BlockDev* __restrict__ tab, StageParams p) {
  const BlockDev& B = tab[blockIdx.y];
  if (!B.implicit) return;
  const VicScratch S = vic_scratch(B);
  const int ng = B.ng, nc1 = B.nc1, n = nc1 - 2 * ng;
  const size_t plane = (size_t)nc1 * B.nc2 * B.nc3;
  const real* uin = static_cast<const real*>(B.buf[p.in]);
  const real* u0 = static_cast<const real*>(B.buf[p.u0]);
  real* uout = static_cast<real*>(B.buf[p.out]);
  const double grav = B.grav1;
  const double vol = B.dx3 * (B.dx2 * B.dx1);
  const double rvol = 1. / vol;
  const double* x1v = B.x1v + ng;
  const double* x1f = B.x1f + ng;
  const size_t cs = S.cells;
  const bool wood = n >= 3;
  const bool partial = B.implicit == 1;
  const real w0 = real(p.w0), w1 = real(p.w1), w2 = real(p.w2);
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < S.cells;
       e += (size_t)gridDim.x * blockDim.x) {
    const size_t col = e / n;
    const int i = (int)(e - col * n);
    const double* D = S.D + col * n * 5;
    const double* du = S.du + col * n;
    const double* du0 = S.du0 + col * n;
    const bool ok = vfinite(D[0]);
    double d[5];
    if (ok) {
      const FinishCol F = finish_col(S, col, n);
      d[0] = du[i] + F.mdn[i];
      d[1] = D[i * 5 + 1];
      if (!partial) {
        d[2] = D[i * 5 + 2];
        d[3] = D[i * 5 + 3];
      } else {
        // vic_tangential_momentum_column: the face below adds its transfer,
        // then the face above takes its own (a zero transfer is skipped)
        const double* vt[2] = {F.vt2, F.vt3};
#pragma unroll
        for (int t = 0; t < 2; ++t) {
          double a = du[(2 + t) * cs + i];
          if (i > 0) {
            const double q = F.mq[i];
            const double pm = q * vt[t][q > 0 ? i - 1 : i];
            if (pm != 0) a += vdiv(pm, vol, rvol);
          }
          if (i + 1 < n) {
            const double q = F.mq[i + 1];
            const double pm = q * vt[t][q > 0 ? i : i + 1];
            if (pm != 0) a -= vdiv(pm, vol, rvol);
          }
          d[2 + t] = a;
        }
      }
      const double projected = vdiv(F.mM[i] - F.mM[i + 1], vol, rvol);
      const double ph = -grav * x1v[i];
      const double pw = ph * (D[i * 5] - du0[i] - projected);
      const double dp_lo = -grav * (x1f[i] - x1v[i]);
      const double dp_hi = -grav * (x1f[i + 1] - x1v[i]);
      const double mv_lo = F.mq[i] - F.mM[i], mv_hi = F.mq[i + 1] - F.mM[i + 1];
      const double cw = vdiv(-(dp_hi * mv_hi - dp_lo * mv_lo), vol, rvol);
      double e4 = D[i * 5 + 4] + (pw + cw);
      if (wood) {
        double wt[3];
        int i0;
        vic_slope_tab(B, n, i, wt, &i0);
        VicK K = vic_krows(B, n, i);
        auto mv = [&](int k) { return (du[k] + F.mdn[k]) - du0[k]; };
        double sl = wt[0] * mv(i0);
        sl += wt[1] * mv(i0 + 1);
        sl += wt[2] * mv(i0 + 2);
        double wk = K.gv * sl;
        auto rw = [&](int k) { return D[k * 5] - du0[k]; };
        double s = K.mid * rw(i);
        if (i >= 1) s += K.lo * rw(i - 1);
        if (i <= n - 2) s += K.hi * rw(i + 1);
        if (i == 0) s += K.t0 * rw(2);
        if (i == n - 1) s += K.t1 * rw(n - 3);
        wk -= s;
        e4 += wk;
      }
      d[4] = e4;
    } else {
#pragma unroll
      for (int v = 0; v < 5; ++v) d[v] = du0[v * cs + i];
    }
    const size_t c = vic_row(B, col) * nc1 + ng + i;
#pragma unroll
    for (int v = 0; v < NHYDRO; ++v) {
      const size_t q = v * plane + c;
      uout[q] = w0 * u0[q] + w1 * uin[q] + w2 * real(d[v]);
    }
  }
}
