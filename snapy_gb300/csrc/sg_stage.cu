// The fused explicit hydro stage of a batch of Cartesian blocks, plus the
// small per-step kernels around it (ghost fill, time step, primitives, redo
// flags).  Compiled twice: SG_REAL=double with -fmad=false (the FP64 parity
// path, bitwise the reference's CPU arithmetic) and SG_REAL=float.
//
// One CTA owns a tile of `tj` x2 columns over the FULL x1 extent (x1 is the
// contiguous vertical axis).  It stages the tile plus its x2 halo as
// primitives in shared memory (one HBM read of the conserved state, U->W on
// the way in), computes every x1 and x2 face flux of the tile in registers
// (WENO5/cp5 face states -> HLLC or LMARS), keeps the fluxes in shared
// memory, and writes  u_out = w0 u0 + w1 u_in + w2 (-dt div F)  for the tile's
// interior cells.  Reference steps fused here (src/hydro/hydro_forward.cpp):
// (1) EOS U->W :340, (2) x1 recon + Riemann :455-664, (3-4) x2 recon +
// Riemann :716-832, wall prescription :664,838, (5) divergence :946-968,
// (6) du = -dt div :983-985, and the RK3 combine of
// src/mesh/meshblock_advance.cpp:329.
#include <cuda_runtime.h>
#include <stdint.h>

#include "sg_device.cuh"
#include "sg_types.h"

#ifndef SG_REAL
#error "compile with -DSG_REAL=double or -DSG_REAL=float"
#endif

#define SG_CAT2(a, b) a##b
#define SG_CAT(a, b) SG_CAT2(a, b)
#ifdef SG_REAL_IS_FLOAT
#define SG_SUFFIX _f32
#else
#define SG_SUFFIX _f64
#endif
#define SG_NAME(x) SG_CAT(x, SG_SUFFIX)

namespace sg {
namespace {

typedef SG_REAL real;
constexpr int kThreads = 256;

__device__ __forceinline__ int find_block(const BlockDev* tab, int nblock,
                                          int tile) {
  int lo = 0, hi = nblock - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (tab[mid].tile0 <= tile)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// the FluxRegister's step-field recursion at one face
// (FluxRegister::end_stage, src/hydro/flux_register.cpp:761-776):
// S <- w1 S + w2 dt T in FP64, the add's alpha form fused as the
// reference's device axpy is (src/utils/step_dt.cu:14-34); at stage 0 the
// field starts from zero (begin_step), so w1 S is +0
__device__ __forceinline__ void step_set(double* s, double t, double w1,
                                         double w2dt, bool first) {
  *s = first ? fma(w2dt, t, 0.) : fma(w2dt, t, *s * w1);
}

// ---- shared-memory staging by 1-D bulk copies (TMA) on an mbarrier ----
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n"
               "fence.mbarrier_init.release.cluster;" ::"r"(smem_u32(bar)),
               "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                   smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n"
      " mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// global -> this CTA's shared memory, `bytes` (a multiple of 16) from two
// 16-byte aligned addresses, completing on `bar`
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src,
                                         uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// the generic-proxy accesses before it are ordered before later bulk copies
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// polls of a staging wait (64 ns apart) before the tile is given up
constexpr int kStagingPolls = 1 << 22;

// face states of 5 consecutive cells: ILT (cp, the -side of the upper face of
// the centre cell) and IRT (cm, the +side of its lower face)
template <bool WENO>
__device__ __forceinline__ real recon_cp(real a, real b, real c, real d,
                                         real e, bool scale) {
  return WENO ? weno5_cp(a, b, c, d, e, scale) : cp5_cp(a, b, c, d, e);
}
template <bool WENO>
__device__ __forceinline__ real recon_cm(real a, real b, real c, real d,
                                         real e, bool scale) {
  return WENO ? weno5_cm(a, b, c, d, e, scale) : cp5_cm(a, b, c, d, e);
}

// left (ILT) and right (IRT) states at a face from a strided line of
// primitives: q points at the cell just above the face (cell f), the stencil
// of ILT is cells f-3..f+1 and of IRT cells f-2..f+2
template <bool SHOCK>
__device__ __forceinline__ void face_states(const real* q, int vstride,
                                            int s, bool scale, real* wl,
                                            real* wr) {
#pragma unroll
  for (int v = 0; v < NHYDRO; ++v) {
    const real* c = q + v * vstride;
    real a = c[-3 * s], b = c[-2 * s], m = c[-s], d = c[0], e = c[s],
         g = c[2 * s];
    if (SHOCK || v == IDN) {
      wl[v] = recon_cp<true>(a, b, m, d, e, scale);
      wr[v] = recon_cm<true>(b, m, d, e, g, scale);
    } else {
      wl[v] = recon_cp<false>(a, b, m, d, e, scale);
      wr[v] = recon_cm<false>(b, m, d, e, g, scale);
    }
  }
}

// nclamp: one more when HLLC's contact pressure was clamped to zero (the
// monitor's riemann.pstar_clamp event, src/riemann/riemann.cpp:330-339)
template <int RK>
__device__ __forceinline__ void riemann(const real* wl, const real* wr,
                                        real gammad, int d, real* flx,
                                        unsigned& nclamp) {
  if (RK == kHllc) {
    real cp;
    hllc_flux<real>(wl, wr, gammad, d, flx, &cp);
    nclamp += cp <= real(0) ? 1u : 0u;
  } else {
    lmars_flux<real>(wl, wr, gammad, d, flx, nullptr);
  }
}

// smem layout of a tile (counts in `real`), shared by the kernel and the
// host-side size query
struct TileLayout {
  int R, ntj, nc1, nx1;
  bool has2, wb, cov, visc;
  int w, f1, f2, ref, pert, cov_arr, divv, vf1, vf2;  // offsets
  int total;
  __host__ __device__ TileLayout(int ntj_, int nc1_, int ng, bool has2_,
                                 bool wb_, bool cov_, bool visc_)
      : ntj(ntj_), nc1(nc1_), has2(has2_), wb(wb_), cov(cov_ && has2_),
        visc(visc_) {
    nx1 = nc1 - 2 * ng;
    int hj = has2 ? ng : 0;
    R = ntj + 2 * hj;
    int o = 0;
    w = o;
    o += NHYDRO * R * nc1;
    f1 = o;
    o += NHYDRO * ntj * (nx1 + 1);
    f2 = o;
    o += has2 ? NHYDRO * (ntj + 1) * nx1 : 0;
    // psf_lo, psf_hi, pref, dref, dsf_l, dsf_r, rho/p per tile row, FP64 in
    // both builds (the FP32 build keeps the hydrostatic reference in FP64)
    constexpr int kDw = (int)(sizeof(double) / sizeof(real));
    o += (o % kDw) ? kDw - (o % kDw) : 0;
    ref = o;
    o += wb ? 7 * ntj * nc1 * kDw : 0;
    pert = o;  // the reconstructed perturbations of p and rho per cell
    o += wb ? 2 * ntj * nc1 : 0;
    cov_arr = o;  // rho, h, un of the x2 face means, x1 rows 0..nc1-1
    o += cov ? 3 * (ntj + 1) * nc1 : 0;
    divv = o;  // div v on tile rows -1..ntj, all x1 cells
    o += visc ? (ntj + 2) * nc1 : 0;
    vf1 = o;  // viscous momentum fluxes, x1 faces
    o += visc ? 3 * ntj * (nx1 + 1) : 0;
    vf2 = o;  // viscous momentum fluxes, x2 faces
    o += (visc && has2) ? 3 * (ntj + 1) * nx1 : 0;
    total = o;
  }
};

// the well-balanced x1 reference of one column (src/hydro/hydro_ref_x1_impl.h
// :20-272 and src/recon/x1_reference.cpp:183-238): one thread runs the
// column's serial face-pressure scan, in the reference's order, so the face
// pressures carry the reference's rounding
// pressure of cell j of a column in FP64: the stored value, plus the base
// where the column holds anomalies (pb non-null)
__device__ __forceinline__ double col_p(const real* pres, const double* pb,
                                        int j) {
  return pb ? as_f64(pres[j]) + pb[j] : as_f64(pres[j]);
}

#ifndef SG_REAL_IS_FLOAT
__device__ __forceinline__ void ref_scan(const real* rho, const real* pres,
                                         const double* pb, int nc1, int iu,
                                         double dx, double grav,
                                         double* psf_lo, double* psf_hi) {
  const double minp = 2.2250738585072014e-308;
  double rdt_top = col_p(pres, pb, iu) / as_f64(rho[iu]);
  double top = col_p(pres, pb, iu) * sg_exp(-grav * 0.5 * dx / rdt_top);
  double face = top;
  for (int i = iu; i >= 0; --i) {
    double dp = grav * as_f64(rho[i]) * dx;
    double lo = face + dp, hi = face;
    psf_lo[i] = lo > minp ? lo : minp;
    psf_hi[i] = hi > minp ? hi : minp;
    face = lo;
  }
  face = top;
  for (int i = iu + 1; i < nc1; ++i) {
    double dp = grav * as_f64(rho[i]) * dx;
    double lo = face, hi = lo - dp;
    psf_lo[i] = lo > minp ? lo : minp;
    psf_hi[i] = hi > minp ? hi : minp;
    face = hi;
  }
}

#endif

__device__ __forceinline__ double wall_rop(double r0, double r1, double k) {
  double q = r0 / r1, qk = k == floor(k) ? q : pow(q, k);
  for (int n = 1; k == floor(k) && n < k; ++n) qk *= q;
  double e = r1 > r0 ? r0 * qk : r0 + k * (r0 - r1);
  return e > 0. ? e : r0;
}

__device__ __forceinline__ double rop_smooth(const double* ropc, int i,
                                             int jlo, int jhi, bool ext_lo,
                                             bool ext_hi) {
  auto rop = [&](int j) { return ropc[j]; };
  if (!(ext_lo && i - 2 < jlo) && !(ext_hi && i + 2 > jhi))
    return rop(i < jlo ? jlo : (i > jhi ? jhi : i));
  double v[5];
#pragma unroll
  for (int m = -2; m <= 2; ++m) {
    int j = i + m;
    if (j < jlo)
      v[m + 2] = ext_lo ? wall_rop(rop(jlo), rop(jlo + 1), (double)(jlo - j))
                        : rop(jlo);
    else if (j > jhi)
      v[m + 2] = ext_hi ? wall_rop(rop(jhi), rop(jhi - 1), (double)(j - jhi))
                        : rop(jhi);
    else
      v[m + 2] = rop(j);
  }
  return (v[0] + 4. * v[1] + 6. * v[2] + 4. * v[3] + v[4]) / 16.;
}

__constant__ double c_w6[6] = {11. / 1440., -31. / 480., 401. / 720.,
                               401. / 720., -31. / 480., 11. / 1440.};
__constant__ double c_w6e[2][6] = {
    {95. / 288., 1427. / 1440., -133. / 240., 241. / 720., -173. / 1440.,
     3. / 160.},
    {-3. / 160., 637. / 1440., 511. / 720., -43. / 240., 77. / 1440.,
     -11. / 1440.}};

// hydro_ref_x1_cell_impl (uniform grid) for cell i of one column
__device__ __forceinline__ void ref_cell(const double* ropc,
                                         const double* psf_lo,
                                         const double* psf_hi, int i, int nc1,
                                         int iu, bool phys_in, bool phys_out,
                                         bool wall_clamp, double* pref,
                                         double* dref, double* dsf) {
  const int il = nc1 - 1 - iu;
  bool thin = (iu - il + 1) < 5, fits = iu >= 4;
  bool wall_in = wall_clamp && phys_in && i >= il && i < il + 2;
  bool wall_out = wall_clamp && phys_out && i > iu - 2 && i <= iu;
  bool clamp_in = wall_in && fits && !(thin && phys_out);
  bool clamp_out = wall_out && fits && !(thin && phys_in);
  double lo = psf_lo[i], hi = psf_hi[i];
  double cell_pref = 0.5 * (lo + hi);
  double lower = lo < hi ? lo : hi, upper = lo > hi ? lo : hi;
  auto face = [&](int f) -> double {
    return f < nc1 ? (double)psf_lo[f] : (double)psf_hi[nc1 - 1];
  };
  auto six = [&](int start, const double* wt, bool rev) {
    double value = 0.;
    for (int m = 0; m < 6; ++m) value += wt[rev ? 5 - m : m] * face(start + m);
    if (value >= lower && value <= upper) cell_pref = value;
  };
  if (i >= 2 && i < nc1 - 2 && !wall_in && !wall_out) six(i - 2, c_w6, false);
  if (clamp_in) six(il, c_w6e[i - il], false);
  if (clamp_out) {
    int s0 = iu + 1 - 5;
    six(s0, c_w6e[4 - (i - s0)], true);
  }
  if (!phys_in && i < 2) six(0, c_w6e[i], false);
  if (!phys_out && i >= nc1 - 2) six(nc1 - 5, c_w6e[4 - (i - (nc1 - 5))], true);
  pref[i] = cell_pref;
  int jlo = (wall_clamp && phys_in) ? il : 0;
  int jhi = (wall_clamp && phys_out) ? iu : nc1 - 1;
  bool ext_lo = wall_clamp && phys_in && il + 1 <= iu;
  bool ext_hi = wall_clamp && phys_out && iu - 1 >= il;
  double rs = rop_smooth(ropc, i, jlo, jhi, ext_lo, ext_hi);
  double rf = rs;
  if (i > 0) rf = 0.5 * (rop_smooth(ropc, i - 1, jlo, jhi, ext_lo, ext_hi) + rs);
  dref[i] = cell_pref * rs;
  dsf[i] = lo * rf;
}

// the six-face stencil ref_cell tries for cell i, if any (at most one
// applies to a cell): its first face, its weight row and its direction
template <typename W6>
__device__ __forceinline__ bool ref_stencil(int i, int nc1, int iu,
                                            bool phys_in, bool phys_out,
                                            bool wall_clamp, const W6* w6,
                                            const W6 (*w6e)[6], int* start,
                                            const W6** wt, bool* rev) {
  const int il = nc1 - 1 - iu;
  const bool thin = (iu - il + 1) < 5, fits = iu >= 4;
  const bool wall_in = wall_clamp && phys_in && i >= il && i < il + 2;
  const bool wall_out = wall_clamp && phys_out && i > iu - 2 && i <= iu;
  *rev = false;
  if (i >= 2 && i < nc1 - 2 && !wall_in && !wall_out) {
    *start = i - 2;
    *wt = w6;
    return true;
  }
  if (wall_in && fits && !(thin && phys_out)) {
    *start = il;
    *wt = w6e[i - il];
    return true;
  }
  if (wall_out && fits && !(thin && phys_in)) {
    const int s0 = iu + 1 - 5;
    *start = s0;
    *wt = w6e[4 - (i - s0)];
    *rev = true;
    return true;
  }
  if (!phys_in && i < 2) {
    *start = 0;
    *wt = w6e[i];
    return true;
  }
  if (!phys_out && i >= nc1 - 2) {
    *start = nc1 - 5;
    *wt = w6e[4 - (i - (nc1 - 5))];
    *rev = true;
    return true;
  }
  return false;
}

#ifdef SG_REAL_IS_FLOAT
// ---------------------------------------------------------------------------
// The FP32 build's well-balanced reference in anomaly form.  The state is
// stored as anomalies about the FP64 base (rho_b, p_b, pf_b), and the
// reference is linear in the face pressures: the scan of a column gives
//   PF(f) = top + sum g dx rho_k = [top_b + sum g dx rho_b,k] + (top - top_b)
//           + sum g dx rho'_k,
// so PF(f) - pf_b(f) = Eb(f) + (top - top_b) + sum g dx rho'_k, with Eb the
// base's own scan less pf_b.  Eb, the base's top face pressure and the base
// parts of the cell pressures (the mid value, the two faces and the stencil,
// each less p_b) are formed in FP64 once per block and stage
// (base_ref_kernel); a tile forms top - top_b once per column in FP64 and the
// rest in FP32 on anomalies, so no FP32 value carries the 1e5 Pa base.  The
// densities stay totals, as in the tile's primitives.
__constant__ float c_w6f[6] = {(float)(11. / 1440.), (float)(-31. / 480.),
                               (float)(401. / 720.), (float)(401. / 720.),
                               (float)(-31. / 480.), (float)(11. / 1440.)};
__constant__ float c_w6ef[2][6] = {
    {(float)(95. / 288.), (float)(1427. / 1440.), (float)(-133. / 240.),
     (float)(241. / 720.), (float)(-173. / 1440.), (float)(3. / 160.)},
    {(float)(-3. / 160.), (float)(637. / 1440.), (float)(511. / 720.),
     (float)(-43. / 240.), (float)(77. / 1440.), (float)(-11. / 1440.)}};

struct RefTab {
  const float *pbf, *pb, *eb, *cmid, *clo, *chi, *cst, *rb, *rr;
  const float* top;  // the base's top face pressure and exp(-c rho_b / p_b)
};

__device__ __forceinline__ RefTab ref_tab(const double* refb, int nc1) {
  const float* t = reinterpret_cast<const float*>(refb + 1);
  RefTab r;
  r.pbf = t;
  r.pb = r.pbf + (nc1 + 1);
  r.eb = r.pb + nc1;
  r.cmid = r.eb + (nc1 + 1);
  r.clo = r.cmid + nc1;
  r.chi = r.clo + nc1;
  r.cst = r.chi + nc1;
  r.rb = r.cst + nc1;
  r.rr = r.rb + nc1;
  r.top = r.rr + nc1;
  return r;
}

// one warp per block
__global__ void __launch_bounds__(32) base_ref_kernel(const BlockDev* tab) {
  const BlockDev& B = tab[blockIdx.x];
  if (!B.refb || !B.base) return;
  const int nc1 = B.nc1, iu = nc1 - 1 - B.ng;
  const int lane = threadIdx.x;
  const unsigned full = 0xffffffffu;
  const double* rb = base_rho(B.base, nc1);
  const double* pb = base_p(B.base, nc1);
  const double* pbf = base_pf(B.base, nc1);
  float* t = reinterpret_cast<float*>(B.refb + 1);
  float* tpbf = t;
  float* tpb = tpbf + (nc1 + 1);
  float* teb = tpb + nc1;
  float* tmid = teb + (nc1 + 1);
  float* tlo = tmid + nc1;
  float* thi = tlo + nc1;
  float* tst = thi + nc1;
  float* trb = tst + nc1;
  float* trr = trb + nc1;
  float* ttop = trr + nc1;
  const double grav = -B.grav1, dx = B.dx1;
  const double ptop = pb[iu];
  const double eb_top = sg_exp(-grav * 0.5 * dx / (ptop / rb[iu]));
  const double top = ptop * eb_top;
  if (lane == 0) {
    B.refb[0] = top;
    ttop[0] = (float)top;
    ttop[1] = (float)eb_top;
  }
  const double* rr = base_r(B.base, nc1);
  // the base's scanned face pressures, ref_scan's sums as warp prefix sums
  double carry = 0.;
  for (int c0 = iu; c0 >= 0; c0 -= 32) {
    const int i = c0 - lane;
    double v = i >= 0 ? grav * rb[i] * dx : 0.;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const double u = __shfl_up_sync(full, v, d);
      if (lane >= d) v += u;
    }
    const double S = carry + v;
    if (i >= 0) teb[i] = (float)((top + S) - pbf[i]);
    carry = __shfl_sync(full, S, 31);
  }
  carry = 0.;
  for (int c0 = iu + 1; c0 <= nc1; c0 += 32) {
    const int f = c0 + lane, k = f - 1;
    double v = (k > iu && k < nc1) ? grav * rb[k] * dx : 0.;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const double u = __shfl_up_sync(full, v, d);
      if (lane >= d) v += u;
    }
    const double S = carry + v;
    if (f <= nc1) teb[f] = (float)((top - S) - pbf[f]);
    carry = __shfl_sync(full, S, 31);
  }
  const bool phys_in = B.bc[0] != kBcNone, phys_out = B.bc[1] != kBcNone;
  for (int i = lane; i <= nc1; i += 32) {
    tpbf[i] = (float)pbf[i];
    if (i == nc1) break;
    tpb[i] = (float)pb[i];
    trb[i] = (float)rb[i];
    trr[i] = (float)rr[i];
    tmid[i] = (float)(0.5 * (pbf[i] + pbf[i + 1]) - pb[i]);
    tlo[i] = (float)(pbf[i] - pb[i]);
    thi[i] = (float)(pbf[i + 1] - pb[i]);
    int s0;
    const double* wt;
    bool rev;
    double c = 0.;
    if (ref_stencil<double>(i, nc1, iu, phys_in, phys_out,
                            B.wb_wall_clamp != 0, c_w6, c_w6e, &s0, &wt,
                            &rev)) {
      for (int m = 0; m < 6; ++m) c += wt[rev ? 5 - m : m] * pbf[s0 + m];
      c -= pb[i];
    }
    tst[i] = (float)c;
  }
}

__device__ __forceinline__ float wall_rop_f(float r0, float r1, float k) {
  float q = r0 / r1, qk = k == floorf(k) ? q : powf(q, k);
  for (int n = 1; k == floorf(k) && n < k; ++n) qk *= q;
  float e = r1 > r0 ? r0 * qk : r0 + k * (r0 - r1);
  return e > 0.f ? e : r0;
}

__device__ __forceinline__ float rop_smooth_f(const float* ropc, int i,
                                              int jlo, int jhi, bool ext_lo,
                                              bool ext_hi) {
  if (!(ext_lo && i - 2 < jlo) && !(ext_hi && i + 2 > jhi))
    return ropc[i < jlo ? jlo : (i > jhi ? jhi : i)];
  float v[5];
#pragma unroll
  for (int m = -2; m <= 2; ++m) {
    const int j = i + m;
    if (j < jlo)
      v[m + 2] = ext_lo ? wall_rop_f(ropc[jlo], ropc[jlo + 1], (float)(jlo - j))
                        : ropc[jlo];
    else if (j > jhi)
      v[m + 2] = ext_hi ? wall_rop_f(ropc[jhi], ropc[jhi - 1], (float)(j - jhi))
                        : ropc[jhi];
    else
      v[m + 2] = ropc[j];
  }
  return (v[0] + 4.f * v[1] + 6.f * v[2] + 4.f * v[3] + v[4]) / 16.f;
}
#endif

// one tile of the batch: `tj` x2 columns of one block over its full x1
template <int RK, bool SHOCK>
__device__ __forceinline__ bool stage_tile(const BlockDev* __restrict__ tab,
                                           const StageParams& p, int tile,
                                           real* sm, uint64_t* bar,
                                           uint32_t& phase, int* fail) {
  const int bi = find_block(tab, p.nblock, tile);
  const BlockDev& B = tab[bi];
  const int nc1 = B.nc1, nc2 = B.nc2, ng = B.ng;
  const int nx1 = nc1 - 2 * ng;
  const bool has2 = nc2 > 1;
  const int hj = has2 ? ng : 0;
  // tile t of the block: x2 strip t % strips of interior x3 plane t / strips
  const int strips = ((has2 ? nc2 - 2 * ng : 1) + B.tj - 1) / B.tj;
  const int t = (tile - B.tile0) % strips;
  const int kk = (tile - B.tile0) / strips;
  const size_t koff = (size_t)(B.nc3 > 1 ? ng + kk : 0) * nc1 * nc2;
  const int j0 = (has2 ? ng : 0) + t * B.tj;
  const int jend = has2 ? nc2 - ng : 1;
  const int ntj = min(B.tj, jend - j0);
  const bool wb = B.grav1 != 0.;
  const bool visc = B.nu_iso > 0.;
  const TileLayout L(ntj, nc1, ng, has2, wb, B.flux_cov != 0 && nc1 >= 3,
                     visc);
  const int R = L.R;
  const size_t plane = (size_t)nc1 * nc2 * B.nc3;
  const real* __restrict__ uin = static_cast<const real*>(B.buf[p.in]);
  const real* __restrict__ u0 = static_cast<const real*>(B.buf[p.u0]);
  real* uout = static_cast<real*>(B.buf[p.out]);
  const real gammad = real(B.gammad);
  const bool scale = p.scale != 0;
  const int il = ng, iu1 = nc1 - ng;  // interior x1 cells il..iu1-1
  const double dt = p.dt[bi];
  unsigned nclamp = 0;  // this thread's HLLC contact-pressure clamps
  // FP32 under gravity: the buffers hold anomalies about the FP64 base
  // (rho_b, 0, 0, 0, e_b)(x1); the tile keeps the total rho and the
  // pressure anomaly p - p_b, and every Riemann solve works on anomalies
  const double* base = B.base;
  const double* rb = base ? base_rho(base, nc1) : nullptr;
  const double* pbc = base ? base_p(base, nc1) : nullptr;
  const double* pbf = base ? base_pf(base, nc1) : nullptr;
  const double* rrb = base ? base_r(base, nc1) : nullptr;
#ifdef SG_REAL_IS_FLOAT
  // the FP32 build reads the base (and the x1 geometry) from its FP32 tables
  const RefTab T = base ? ref_tab(B.refb, nc1) : RefTab{};
  auto rb_r = [&](int i) -> real { return T.rb[i]; };
  auto pb_r = [&](int i) -> real { return T.pb[i]; };
  auto rr_r = [&](int i) -> real { return T.rr[i]; };
  auto xt_r = [&](int k, int q) -> real { return B.x1tab32[8 * k + q]; };
  // (the covariance row also runs without gravity, where there is no table)
  auto covdx_r = [&](int i) -> real {
    return B.x1tab32 ? B.x1tab32[8 * (i - ng) + 6]
                     : real(B.x1v[i + 1] - B.x1v[i - 1]);
  };
#else
  auto rb_r = [&](int i) -> real { return real(rb[i]); };
  auto pb_r = [&](int i) -> real { return real(pbc[i]); };
  auto rr_r = [&](int i) -> real { return real(rrb[i]); };
  auto xt_r = [&](int k, int q) -> real { return real(B.x1tab[6 * k + q]); };
  auto covdx_r = [&](int i) -> real { return real(B.x1v[i + 1] - B.x1v[i - 1]); };
#endif

  const int wstride = R * nc1;  // one variable of the W tile
  real* W = sm + L.w;
  const int nf1 = nx1 + 1;
  real* F1 = sm + L.f1;
  const int f1stride = ntj * nf1;
  real* F2 = sm + L.f2;
  const int f2stride = (ntj + 1) * nx1;

  // (1) the tile and its x2 halo, U -> W.  The R rows of a variable are one
  // contiguous span of R nc1 values; where every span starts and ends on 16
  // bytes, one thread stages the five spans by bulk copies (TMA) into W and
  // the tile converts in place, else every thread loads its cells
  const size_t row0 = koff + (size_t)(j0 - hj) * nc1;
  const uint32_t span = (uint32_t)(R * nc1 * sizeof(real));
  const bool bulk =
      span % 16 == 0 && (plane * sizeof(real)) % 16 == 0 &&
      (reinterpret_cast<uintptr_t>(uin + row0) % 16) == 0;
  if (bulk) {
    if (threadIdx.x == 0) {
      fence_proxy_async();  // the previous tile's reads of W come first
      mbar_expect_tx(bar, NHYDRO * span);
#pragma unroll
      for (int v = 0; v < NHYDRO; ++v)
        bulk_g2s(W + v * wstride, uin + v * plane + row0, span, bar);
      bool ok = false;
      for (int it = 0; it < kStagingPolls; ++it) {
        if (mbar_test(bar, phase)) {
          ok = true;
          break;
        }
        __nanosleep(64);
      }
      if (!ok) {
        // give the tile up: flag the block, then wait (bounded again) for
        // the copies still in flight before the CTA leaves
        atomicOr(&p.status[bi], kStatusStaging);
        for (int it = 0; it < kStagingPolls && !mbar_test(bar, phase); ++it)
          __nanosleep(1024);
      }
      *fail = ok ? 0 : 1;
    }
    __syncthreads();
    phase ^= 1u;
    if (*fail) return false;
    for (int idx = threadIdx.x; idx < R * nc1; idx += blockDim.x) {
      real uc[NHYDRO], wc[NHYDRO];
#pragma unroll
      for (int v = 0; v < NHYDRO; ++v) uc[v] = W[v * wstride + idx];
      if (rb) uc[IDN] = rb_r(idx % nc1) + uc[IDN];
      cons2prim<real>(uc, wc, gammad);
#pragma unroll
      for (int v = 0; v < NHYDRO; ++v) W[v * wstride + idx] = wc[v];
    }
  } else {
    for (int idx = threadIdx.x; idx < R * nc1; idx += blockDim.x) {
      real uc[NHYDRO], wc[NHYDRO];
#pragma unroll
      for (int v = 0; v < NHYDRO; ++v) uc[v] = uin[v * plane + row0 + idx];
      // with a base: rho_b + rho', and p' = (g - 1)(E' - ke) since p_b is
      // (g - 1) e_b
      if (rb) uc[IDN] = rb_r(idx % nc1) + uc[IDN];
      cons2prim<real>(uc, wc, gammad);
#pragma unroll
      for (int v = 0; v < NHYDRO; ++v) W[v * wstride + idx] = wc[v];
    }
  }
  __syncthreads();

  // (2) the well-balanced x1 reference of each tile column
  double* REF = reinterpret_cast<double*>(sm + L.ref);
  const int rs_ = ntj * nc1;  // one reference array of the tile
  const bool phys_in = B.bc[0] != kBcNone, phys_out = B.bc[1] != kBcNone;
  const int iu = nc1 - 1 - ng;
  real* PP = sm + L.pert;  // p - pref of each tile cell
  real* PD = PP + rs_;     // rho - dref
#ifdef SG_REAL_IS_FLOAT
  // the FP32 reference (anomalies of the face and cell pressures about the
  // base, densities as totals), in the reference region as floats: per
  // column PFa [nc1 + 1] (face pressure - pf_b), rop, pref' (cell pressure
  // - p_b), dref, dsf_l, dsf_r
  float* RF = reinterpret_cast<float*>(REF);
  const int cs1 = nc1 + 1, rsf = ntj * cs1;
  if (wb) {
    const float gdx = (float)(-B.grav1 * B.dx1);
    const float cg = 0.5f * gdx;  // g dx / 2
    // a warp per column: top - top_b in FP64, then the anomalies' prefix
    // sums of g dx rho' (the stored density anomalies) in FP32
    for (int jt = threadIdx.x >> 5; jt < ntj; jt += blockDim.x >> 5) {
      const int lane = threadIdx.x & 31;
      const unsigned full = 0xffffffffu;
      const real* ra = uin + row0 + (size_t)(hj + jt) * nc1;
      const real* pres = W + IPR * wstride + (hj + jt) * nc1;
      float* PFa = RF + jt * cs1;
      // top - top_b, top = p exp(-c rho / p) at the top cell, in FP32 on the
      // anomalies: with x = -c (rho' p_b - rho_b p') / (p_b (p_b + p')),
      // top - top_b = top_b expm1(x) + E_b p' (1 + expm1(x))
      const float pbt = T.pb[iu], rbt = T.rb[iu];
      const float pa = pres[iu], rhoa = ra[iu];
      const float x = -cg * (rhoa * pbt - rbt * pa) / (pbt * (pbt + pa));
      const float em = expm1f(x);
      const float tp = T.top[0] * em + T.top[1] * pa * (1.f + em);
      float carry = 0.f;
      for (int c0 = iu; c0 >= 0; c0 -= 32) {
        const int i = c0 - lane;
        float v = i >= 0 ? gdx * ra[i] : 0.f;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const float u = __shfl_up_sync(full, v, d);
          if (lane >= d) v += u;
        }
        const float S = carry + v;  // over cells i..iu
        if (i >= 0) PFa[i] = (tp + S) + T.eb[i];
        carry = __shfl_sync(full, S, 31);
      }
      carry = 0.f;
      for (int c0 = iu + 1; c0 <= nc1; c0 += 32) {
        const int f = c0 + lane, k = f - 1;
        float v = (k > iu && k < nc1) ? gdx * ra[k] : 0.f;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const float u = __shfl_up_sync(full, v, d);
          if (lane >= d) v += u;
        }
        const float S = carry + v;  // over cells iu+1..f-1
        if (f <= nc1) PFa[f] = (tp - S) + T.eb[f];
        carry = __shfl_sync(full, S, 31);
      }
    }
    // rho / p of every cell once (totals: p = p_b + p')
    for (int idx = threadIdx.x; idx < ntj * nc1; idx += blockDim.x) {
      const int jt = idx / nc1, i = idx - jt * nc1;
      const real* rho = W + IDN * wstride + (hj + jt) * nc1;
      const real* pres = W + IPR * wstride + (hj + jt) * nc1;
      RF[rsf + jt * cs1 + i] = rho[i] / (T.pb[i] + pres[i]);
    }
    __syncthreads();
    // ref_cell on the anomalies: the mid value, the faces and the stencil
    // relative to p_b (their base parts from the table)
    const bool wclamp = B.wb_wall_clamp != 0;
    const int jlo = (wclamp && phys_in) ? il : 0;
    const int jhi = (wclamp && phys_out) ? iu : nc1 - 1;
    const bool ext_lo = wclamp && phys_in && il + 1 <= iu;
    const bool ext_hi = wclamp && phys_out && iu - 1 >= il;
    for (int idx = threadIdx.x; idx < ntj * nc1; idx += blockDim.x) {
      const int jt = idx / nc1, i = idx - jt * nc1;
      const float* PFa = RF + jt * cs1;
      const float* rop = RF + rsf + jt * cs1;
      const float lo = PFa[i] + T.clo[i], hi = PFa[i + 1] + T.chi[i];
      const float lower = fminf(lo, hi), upper = fmaxf(lo, hi);
      float cell = 0.5f * (PFa[i] + PFa[i + 1]) + T.cmid[i];
      int s0;
      const float* wt;
      bool rev;
      if (ref_stencil<float>(i, nc1, iu, phys_in, phys_out, wclamp, c_w6f,
                             c_w6ef, &s0, &wt, &rev)) {
        float value = 0.f;
        for (int m = 0; m < 6; ++m) value += wt[rev ? 5 - m : m] * PFa[s0 + m];
        value += T.cst[i];
        if (value >= lower && value <= upper) cell = value;
      }
      const float rs = rop_smooth_f(rop, i, jlo, jhi, ext_lo, ext_hi);
      const float rf =
          i > 0 ? 0.5f * (rop_smooth_f(rop, i - 1, jlo, jhi, ext_lo, ext_hi) + rs)
                : rs;
      RF[2 * rsf + jt * cs1 + i] = cell;
      RF[3 * rsf + jt * cs1 + i] = (T.pb[i] + cell) * rs;
      RF[4 * rsf + jt * cs1 + i] = (T.pbf[i] + PFa[i]) * rf;
    }
    __syncthreads();
    // dsf_lr: the cp5 rows on dref guarded by the two cells' range, a
    // reflecting wall face the mean of its sides; then PP, PD
    for (int idx = threadIdx.x; idx < ntj * nc1; idx += blockDim.x) {
      const int jt = idx / nc1, f = idx - jt * nc1;
      const float* dref = RF + 3 * rsf + jt * cs1;
      float* DL = RF + 4 * rsf + jt * cs1;
      float* DR = RF + 5 * rsf + jt * cs1;
      const float dsf = DL[f];
      float l = dsf, r = dsf;
      if (nc1 >= 6 && f >= 2 && f <= nc1 - 2) {
        const float a = dref[f - 1], c = dref[f];
        const float lo = fminf(a, c), hi = fmaxf(a, c);
        if (f <= nc1 - 3) {
          const float lin = cp5_cm<float>(dref[f - 2], dref[f - 1], dref[f],
                                          dref[f + 1], dref[f + 2]);
          if (lin >= lo && lin <= hi) r = lin;
        }
        if (f >= 3) {
          const float lin = cp5_cp<float>(dref[f - 3], dref[f - 2], dref[f - 1],
                                          dref[f], dref[f + 1]);
          if (lin >= lo && lin <= hi) l = lin;
        }
        if ((f == il && B.bc[0] == kBcReflecting) ||
            (f == iu + 1 && B.bc[1] == kBcReflecting)) {
          const float mean = 0.5f * (l + r);
          l = r = mean;
        }
      }
      DL[f] = l;
      DR[f] = r;
      const real* rho = W + IDN * wstride + (hj + jt) * nc1;
      const real* pres = W + IPR * wstride + (hj + jt) * nc1;
      PP[idx] = pres[f] - RF[2 * rsf + jt * cs1 + f];
      PD[idx] = rho[f] - dref[f];
    }
    __syncthreads();
  }
#else
  if (wb) {
    for (int jt = threadIdx.x; jt < ntj; jt += blockDim.x) {
      const real* rho = W + IDN * wstride + (hj + jt) * nc1;
      const real* pres = W + IPR * wstride + (hj + jt) * nc1;
      ref_scan(rho, pres, pbc, nc1, iu, B.dx1, -B.grav1,
               REF + 0 * rs_ + jt * nc1, REF + 1 * rs_ + jt * nc1);
    }
    // rho / p of every cell once (rop_smooth reads up to five per cell)
    for (int idx = threadIdx.x; idx < ntj * nc1; idx += blockDim.x) {
      const int jt = idx / nc1, i = idx - jt * nc1;
      const real* rho = W + IDN * wstride + (hj + jt) * nc1;
      const real* pres = W + IPR * wstride + (hj + jt) * nc1;
      REF[6 * rs_ + idx] = as_f64(rho[i]) / col_p(pres, pbc, i);
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < ntj * nc1; idx += blockDim.x) {
      const int jt = idx / nc1, i = idx - jt * nc1;
      ref_cell(REF + 6 * rs_ + jt * nc1, REF + jt * nc1, REF + rs_ + jt * nc1,
               i, nc1, iu, phys_in, phys_out, B.wb_wall_clamp != 0,
               REF + 2 * rs_ + jt * nc1, REF + 3 * rs_ + jt * nc1,
               REF + 4 * rs_ + jt * nc1 /* dsf, becomes dsf_l */);
    }
    __syncthreads();
    // dsf_lr: the cp5 row on dref guarded by the two cells' range; a
    // reflecting wall face takes the mean of its two sides.  Face f reads
    // dsf[f] alone, so the ILT side overwrites dsf in place (slot 4); the
    // IRT side goes to slot 5
    for (int idx = threadIdx.x; idx < ntj * nc1; idx += blockDim.x) {
      const int jt = idx / nc1, f = idx - jt * nc1;
      const double* dref = REF + 3 * rs_ + jt * nc1;
      double* DL = REF + 4 * rs_ + jt * nc1;
      double* DR = REF + 5 * rs_ + jt * nc1;
      double dsf = DL[f];
      double l = dsf, r = dsf;
      if (nc1 >= 6 && f >= 2 && f <= nc1 - 2) {
        double a = dref[f - 1], c = dref[f];
        double lo = a < c ? a : c, hi = a > c ? a : c;
        if (f <= nc1 - 3) {
          double lin = cp5_cm<double>(dref[f - 2], dref[f - 1], dref[f],
                                      dref[f + 1], dref[f + 2]);
          if (lin >= lo && lin <= hi) r = lin;
        }
        if (f >= 3) {
          double lin = cp5_cp<double>(dref[f - 3], dref[f - 2], dref[f - 1],
                                      dref[f], dref[f + 1]);
          if (lin >= lo && lin <= hi) l = lin;
        }
        if ((f == il && B.bc[0] == kBcReflecting) ||
            (f == iu + 1 && B.bc[1] == kBcReflecting)) {
          double mean = 0.5 * (l + r);
          l = r = mean;
        }
      }
      DL[f] = l;
      DR[f] = r;
      // the perturbations the x1 reconstruction reads, once per cell
      const real* rho = W + IDN * wstride + (hj + jt) * nc1;
      const real* pres = W + IPR * wstride + (hj + jt) * nc1;
      PP[idx] = real(col_p(pres, pbc, f) - REF[2 * rs_ + idx]);
      PD[idx] = real(as_f64(rho[f]) - REF[3 * rs_ + idx]);
    }
    __syncthreads();
  }
#endif

  // (3) x1 faces il..iu1 of the tile rows; with gravity the face states are
  // the reference plus the reconstructed perturbation (WellBalancedX1)
  for (int idx = threadIdx.x; idx < ntj * nf1; idx += blockDim.x) {
    const int jt = idx / nf1, fi = idx - jt * nf1;
    const int f = il + fi;
    const real* q = W + (hj + jt) * nc1 + f;
    real wl[NHYDRO], wr[NHYDRO], flx[NHYDRO];
    if (!wb) {
      face_states<SHOCK>(q, wstride, 1, scale, wl, wr);
    } else {
      // the perturbation of p (v = IPR) and rho (v = IDN) at cell c, even-
      // mirrored into the x1 wall ghosts
      auto pert = [&](int v, int c) -> real {
        if (c < il && phys_in) c = 2 * il - 1 - c;
        if (c >= iu1 && phys_out) c = 2 * iu1 - 1 - c;
        return (v == IPR ? PP : PD)[jt * nc1 + c];
      };
#pragma unroll
      for (int v = 0; v < NHYDRO; ++v) {
        real s[6];
        if (v == IPR || v == IDN) {
#pragma unroll
          for (int k = 0; k < 6; ++k) s[k] = pert(v, f - 3 + k);
        } else {
#pragma unroll
          for (int k = 0; k < 6; ++k) s[k] = q[v * wstride + k - 3];
        }
        if (SHOCK || v == IDN) {
          wl[v] = weno5_cp(s[0], s[1], s[2], s[3], s[4], scale);
          wr[v] = weno5_cm(s[1], s[2], s[3], s[4], s[5], scale);
        } else {
          wl[v] = cp5_cp(s[0], s[1], s[2], s[3], s[4]);
          wr[v] = cp5_cm(s[1], s[2], s[3], s[4], s[5]);
        }
      }
#ifdef SG_REAL_IS_FLOAT
      // the face pressure's anomaly about pf_b: the reconstructed
      // perturbation plus the reference's anomaly (a total at or below zero
      // takes the reference); the density a total
      const float psfa = RF[jt * cs1 + f], pbff = T.pbf[f];
      float pl = wl[IPR] + psfa, pr = wr[IPR] + psfa;
      wl[IPR] = pl + pbff > 0.f ? pl : psfa;
      wr[IPR] = pr + pbff > 0.f ? pr : psfa;
      real dl = wl[IDN] + RF[4 * rsf + jt * cs1 + f];
      real dr = wr[IDN] + RF[5 * rsf + jt * cs1 + f];
#else
      // the totals in FP64; the Riemann solve takes the anomaly about the
      // base face pressure where there is a base
      const double psf = REF[0 * rs_ + jt * nc1 + f];
      double pl = as_f64(wl[IPR]) + psf, pr = as_f64(wr[IPR]) + psf;
      pl = pl > 0. ? pl : psf;
      pr = pr > 0. ? pr : psf;
      wl[IPR] = real(pbf ? pl - pbf[f] : pl);
      wr[IPR] = real(pbf ? pr - pbf[f] : pr);
      real dl = real(as_f64(wl[IDN]) + REF[4 * rs_ + jt * nc1 + f]);
      real dr = real(as_f64(wr[IDN]) + REF[5 * rs_ + jt * nc1 + f]);
#endif
      const real* rho = W + IDN * wstride + (hj + jt) * nc1;
      wl[IDN] = dl > real(0) ? dl : rho[f > 0 ? f - 1 : 0];
      wr[IDN] = dr > real(0) ? dr : rho[f];
    }
    if (pbf)
#ifdef SG_REAL_IS_FLOAT
      lmars_flux_anom<real>(wl, wr, gammad, 1, T.pbf[f], flx);
#else
      lmars_flux_anom<real>(wl, wr, gammad, 1, real(pbf[f]), flx);
#endif
    else
      riemann<RK>(wl, wr, gammad, 1, flx, nclamp);
    if ((fi == 0 && B.bc[0] == kBcReflecting) ||
        (fi == nx1 && B.bc[1] == kBcReflecting))
      flx[IDN] = flx[IPR] = real(0);
#pragma unroll
    for (int v = 0; v < NHYDRO; ++v) F1[v * f1stride + idx] = flx[v];
  }

  // (4) x2 faces j0..j0+ntj: the Riemann flux on the x1-interior cells and,
  // with the covariance row, the face means on x1 rows 1..nc1-2
  real* COV = sm + L.cov_arr;
  const int cstride = (ntj + 1) * nc1;
  if (has2) {
    const int r0 = L.cov ? 1 : il, r1 = L.cov ? nc1 - 1 : iu1;
    const int nr = r1 - r0;
    for (int idx = threadIdx.x; idx < (ntj + 1) * nr; idx += blockDim.x) {
      const int jf = idx / nr, i = r0 + (idx - jf * nr);
      const real* q = W + (hj + jf) * nc1 + i;
      real wl[NHYDRO], wr[NHYDRO], flx[NHYDRO];
      face_states<SHOCK>(q, wstride, nc1, scale, wl, wr);
      if (L.cov) {
        real wb_[NHYDRO];
#pragma unroll
        for (int v = 0; v < NHYDRO; ++v) wb_[v] = real(0.5) * (wl[v] + wr[v]);
        real pbar = wb_[IPR];
        if (pbc) pbar = pb_r(i) + pbar;  // the total
        real enth = pbar / (gammad - real(1)) + pbar;
        COV[0 * cstride + jf * nc1 + i] = wb_[IDN];
        COV[1 * cstride + jf * nc1 + i] = enth / wb_[IDN];
        COV[2 * cstride + jf * nc1 + i] = wb_[IVY];
      }
      if (i >= il && i < iu1) {
        if (pbc)
          lmars_flux_anom<real>(wl, wr, gammad, 2, pb_r(i), flx);
        else {
          // a tile's last face is the next tile's first: counted there
          unsigned c = 0;
          riemann<RK>(wl, wr, gammad, 2, flx, c);
          if (jf < ntj || j0 + ntj == jend) nclamp += c;
        }
#pragma unroll
        for (int v = 0; v < NHYDRO; ++v)
          F2[v * f2stride + jf * nx1 + (i - il)] = flx[v];
      }
    }
  }

  // div v for the viscous stress: tile rows -1..ntj, x1 cells il-1..iu1
  real* DIVV = sm + L.divv;
  if (visc) {
    // without x2 only the tile row itself (rr = 1) is needed
    const int rlo = has2 ? 0 : 1, nr = has2 ? ntj + 2 : 1, nci = nx1 + 2;
    // quotients by a shared divisor divide through its reciprocal (vdiv:
    // the same bits)
    const real d1 = real(2.) * real(B.dx1), d2 = real(2.) * real(B.dx2);
    const real rd1 = real(1.) / d1, rd2 = real(1.) / d2;
    for (int idx = threadIdx.x; idx < nr * nci; idx += blockDim.x) {
      const int rr = rlo + idx / nci, i = il - 1 + (idx - (rr - rlo) * nci);
      const int r = hj + rr - 1;  // W row
      if (B.visc3) {  // 3-D: the whole divergence, its x3 term included
        DIVV[rr * nc1 + i] = static_cast<const real*>(B.visc3)[
            koff + (size_t)(j0 + rr - 1) * nc1 + i];
        continue;
      }
      const real* vx = W + IVX * wstride + r * nc1;
      real dv = real(0);
      dv += vdiv(vx[i + 1] - vx[i - 1], d1, rd1);
      if (has2) {
        const real* vy = W + IVY * wstride;
        dv += vdiv(vy[(r + 1) * nc1 + i] - vy[(r - 1) * nc1 + i], d2, rd2);
      }
      DIVV[rr * nc1 + i] = dv;
    }
  }
  __syncthreads();

  // (5) the x2 covariance row, then the x2 wall faces
  if (has2) {
    const real s2 = real(B.dx1 * B.dx1 / 12.);
    for (int idx = threadIdx.x; idx < (ntj + 1) * nx1; idx += blockDim.x) {
      const int jf = idx / nx1, ii = idx - jf * nx1, i = il + ii;
      if (L.cov) {
        real dx1 = covdx_r(i);
        const real* rho = COV + jf * nc1;
        const real* h = COV + cstride + jf * nc1;
        const real* un = COV + 2 * cstride + jf * nc1;
        real s2rho = s2 * rho[i];
        const real rdx1 = real(1.) / dx1;
        real d1h = vdiv(h[i + 1] - h[i - 1], dx1, rdx1);
        real dun = vdiv(un[i + 1] - un[i - 1], dx1, rdx1);
        F2[IPR * f2stride + idx] += s2rho * d1h * dun;
      }
      const int jface = j0 + jf;
      if ((jface == ng && B.bc[2] == kBcReflecting) ||
          (jface == nc2 - ng && B.bc[3] == kBcReflecting))
        F2[IDN * f2stride + idx] = F2[IPR * f2stride + idx] = real(0);
    }
  }
  // viscous fluxes (src/forcing/diffusion.cpp:553-683): the momentum rows
  // into VF1/VF2, the energy row posted into the totals
  real* VF1 = sm + L.vf1;
  real* VF2 = sm + L.vf2;
  if (visc) {
    const real nu = real(B.nu_iso);
    const real dx1 = real(B.dx1), dx2 = real(B.dx2);
    const real rdx1 = real(1.) / dx1, rdx2 = real(1.) / dx2;
    const real d2x1 = real(2.) * dx1, d2x2 = real(2.) * dx2;
    const real rd2x1 = real(1.) / d2x1, rd2x2 = real(1.) / d2x2;
    const real* vx = W + IVX * wstride;
    const real* vy = W + IVY * wstride;
    const real* vz = W + IVZ * wstride;
    const real* rho = W + IDN * wstride;
    const bool wlo = B.bc[0] == kBcReflecting, whi = B.bc[1] == kBcReflecting;
    for (int idx = threadIdx.x; idx < ntj * nf1; idx += blockDim.x) {
      const int jt = idx / nf1, fi = idx - jt * nf1, f = il + fi;
      const int r = hj + jt;
      const int o = r * nc1;
      real rf = real(0.5) * (rho[o + f] + rho[o + f - 1]);
      if (nf1 >= 3) {
        real tt = dx1 / (dx1 + dx1);
        if (f == il && wlo) {
          real vn = rho[o + il], vq = rho[o + il + 1];
          real wall = (real(1.) + tt) * vn - tt * vq;
          rf = wall > real(0) ? wall : vn;
        }
        if (f == iu1 && whi) {
          real vn = rho[o + iu1 - 1], vq = rho[o + iu1 - 2];
          real wall = (real(1.) + tt) * vn - tt * vq;
          rf = wall > real(0) ? wall : vn;
        }
      }
      const real* dvr = DIVV + (jt + 1) * nc1;
      real divf = real(0.5) * (dvr[f] + dvr[f - 1]);
      real e = real(0);
#pragma unroll
      for (int ivar = 0; ivar < 3; ++ivar) {
        const real* vc = ivar == 0 ? vx : (ivar == 1 ? vy : vz);
        real stress = vdiv(vc[o + f] - vc[o + f - 1], dx1, rdx1);
        if (ivar == 0) {
          stress = real(2.) * stress - real(2. / 3.) * divf;
        } else if (ivar == 1 && has2) {
          real below = vdiv(vx[o + nc1 + f - 1] - vx[o - nc1 + f - 1], d2x2, rd2x2);
          real above = vdiv(vx[o + nc1 + f] - vx[o - nc1 + f], d2x2, rd2x2);
          stress += real(0.5) * (above + below);
        } else if (ivar == 2 && B.visc3) {  // 3-D: dv1/dx3 of the two cells
          const real* d31 = static_cast<const real*>(B.visc3) + plane +
                            koff + (size_t)(j0 + jt) * nc1;
          stress += real(0.5) * (d31[f] + d31[f - 1]);
        }
        real mf = -nu * rf * stress;
        VF1[ivar * f1stride + idx] = mf;
        e += real(0.5) * (vc[o + f] + vc[o + f - 1]) * mf;
      }
      F1[IPR * f1stride + idx] += e;
      if ((fi == 0 && wlo) || (fi == nx1 && whi))
        F1[IDN * f1stride + idx] = F1[IPR * f1stride + idx] = real(0);
    }
    if (has2) {
      for (int idx = threadIdx.x; idx < (ntj + 1) * nx1; idx += blockDim.x) {
        const int jf = idx / nx1, ii = idx - jf * nx1, i = il + ii;
        const int r = hj + jf;  // the cell above face jf
        const int o = r * nc1, om = (r - 1) * nc1;
        real rf = real(0.5) * (rho[o + i] + rho[om + i]);
        const real* dva = DIVV + (jf + 1) * nc1;
        const real* dvb = DIVV + jf * nc1;
        real divf = real(0.5) * (dva[i] + dvb[i]);
        real e = real(0);
#pragma unroll
        for (int ivar = 0; ivar < 3; ++ivar) {
          const real* vc = ivar == 0 ? vx : (ivar == 1 ? vy : vz);
          real stress = vdiv(vc[o + i] - vc[om + i], dx2, rdx2);
          if (ivar == 1) {
            stress = real(2.) * stress - real(2. / 3.) * divf;
          } else if (ivar == 0) {
            real below = vdiv(vy[om + i + 1] - vy[om + i - 1], d2x1, rd2x1);
            real above = vdiv(vy[o + i + 1] - vy[o + i - 1], d2x1, rd2x1);
            stress += real(0.5) * (above + below);
          } else if (ivar == 2 && B.visc3) {  // 3-D: dv2/dx3 of the two cells
            const real* d32 = static_cast<const real*>(B.visc3) + 2 * plane +
                              koff + i;
            stress += real(0.5) * (d32[(size_t)(j0 + jf) * nc1] +
                                   d32[(size_t)(j0 + jf - 1) * nc1]);
          }
          real mf = -nu * rf * stress;
          VF2[ivar * f2stride + idx] = mf;
          e += real(0.5) * (vc[o + i] + vc[om + i]) * mf;
        }
        F2[IPR * f2stride + idx] += e;
        const int jface = j0 + jf;
        if ((jface == ng && B.bc[2] == kBcReflecting) ||
            (jface == nc2 - ng && B.bc[3] == kBcReflecting))
          F2[IDN * f2stride + idx] = F2[IPR * f2stride + idx] = real(0);
      }
    }
  }
  __syncthreads();

  // the stage's face totals T_1, T_2 are final here: the FluxRegister's
  // step fields (FP64; under a base the normal-momentum row gets the base
  // face pressure back).  An implicit block stages T_1 for the solve's
  // posts, which its finish kernel adds before the recursion.  Each face
  // has one writer: x2 faces shared by two tiles go to the upper tile,
  // except the block's last face
  if (B.step[0] || B.step[1]) {
    const double w1s = p.w1, w2dt = p.w2 * dt;
    const bool first = p.first != 0;
    const size_t nx2i = has2 ? nc2 - 2 * ng : 1;
    if (double* S1 = B.step[0]) {
      const size_t ncols = nx2i * (B.nc3 > 1 ? B.nc3 - 2 * ng : 1);
      for (int idx = threadIdx.x; idx < ntj * nf1; idx += blockDim.x) {
        const int jt = idx / nf1, fi = idx - jt * nf1, f = il + fi;
        const size_t col = (size_t)kk * nx2i + (j0 + jt - hj);
        const size_t c = koff + (size_t)(j0 + jt) * nc1 + f;
#pragma unroll
        for (int v = 0; v < NHYDRO; ++v) {
          double t = as_f64(F1[v * f1stride + idx]);
          if (pbf && v == IVX) t = t + pbf[f];
          if (B.implicit)
            B.t1[((size_t)v * ncols + col) * nf1 + fi] = t;
          else
            step_set(S1 + v * plane + c, t, w1s, w2dt, first);
        }
      }
    }
    if (double* S2 = B.step[1]) {
      for (int idx = threadIdx.x; idx < (ntj + 1) * nx1; idx += blockDim.x) {
        const int jf = idx / nx1, i = il + (idx - jf * nx1);
        if (jf == ntj && j0 + ntj != jend) continue;
        const size_t c = koff + (size_t)(j0 + jf) * nc1 + i;
#pragma unroll
        for (int v = 0; v < NHYDRO; ++v) {
          double t = as_f64(F2[v * f2stride + idx]);
          if (pbc && v == IVY) t = t + pbc[i];
          step_set(S2 + v * plane + c, t, w1s, w2dt, first);
        }
      }
    }
  }

  // passive scalars ride on the stage's mass flux (the register's mass row,
  // walls prescribed): every face of the tile's interior cells, FP64, with
  // the step fields' one writer per face
  if (B.nscalar > 0) {
    for (int idx = threadIdx.x; idx < ntj * nf1; idx += blockDim.x) {
      const int jt = idx / nf1, fi = idx - jt * nf1, f = il + fi;
      B.mflux[0][koff + (size_t)(j0 + jt) * nc1 + f] =
          as_f64(F1[IDN * f1stride + idx]);
    }
    if (has2) {
      for (int idx = threadIdx.x; idx < (ntj + 1) * nx1; idx += blockDim.x) {
        const int jf = idx / nx1, i = il + (idx - jf * nx1);
        if (jf == ntj && j0 + ntj != jend) continue;
        B.mflux[1][koff + (size_t)(j0 + jf) * nc1 + i] =
            as_f64(F2[IDN * f2stride + idx]);
      }
    }
  }

  // (6) divergence, du = -dt div, gravity, viscous momentum, the x1 gravity
  // energy correction, and the RK combine on the interior cells
  const real a1 = real(B.dx3 * B.dx2), a2 = real(B.dx3 * B.dx1);
  const real vol = real(B.dx3 * (B.dx2 * B.dx1));
  const real rvol = real(1.) / vol;  // every quotient by vol divides by it
  const real rdt = real(dt), mdt = real(-dt);
  const real w0 = real(p.w0), w1 = real(p.w1), w2 = real(p.w2);
  const real g = real(B.grav1);
  for (int idx = threadIdx.x; idx < ntj * nx1; idx += blockDim.x) {
    const int jt = idx / nx1, ii = idx - jt * nx1;
    const int i = il + ii;
    const size_t c = koff + (size_t)(j0 + jt) * nc1 + i;
    const int wc = (hj + jt) * nc1 + i;
    // the cell's index among the interior cells (the implicit solve's and
    // the x3 differences' layout)
    const size_t nx2i = has2 ? nc2 - 2 * ng : 1;
    const size_t icells = (size_t)nx1 * nx2i * (B.nc3 > 1 ? B.nc3 - 2 * ng : 1);
    const size_t vci = ((size_t)kk * nx2i + (j0 + jt - (has2 ? ng : 0))) * nx1 + ii;
    const real* dv3 = static_cast<const real*>(B.dv3);
    real du[NHYDRO];
#pragma unroll
    for (int v = 0; v < NHYDRO; ++v) {
      const real* f1 = F1 + v * f1stride + jt * nf1 + ii;
      real dv = a1 * f1[1] - a1 * f1[0];
      if (has2) {
        const real* f2 = F2 + v * f2stride + jt * nx1 + ii;
        dv = dv + (a2 * f2[nx1] - a2 * f2[0]);
      }
      if (dv3) dv = dv + dv3[v * icells + vci];
      du[v] = mdt * vdiv(dv, vol, rvol);
    }
    if (wb) {
      const real rho = W[IDN * wstride + wc], vx = W[IVX * wstride + wc];
      if (rrb) {
        // the x1 fluxes carried p* - pf_b: the base's face-pressure
        // difference and weight balance to r_b (FP64), which leaves the
        // anomaly's weight rho' g
        const real rho_a = uin[IDN * plane + c];
        du[IVX] += rdt * rho_a * g + rdt * rr_r(i);
      } else {
        du[IVX] += rdt * rho * g * real(1.);
      }
      du[IPR] += rdt * rho * vx * g * real(1.);
    }
    if (visc) {
      // the momentum rows (IDN has no viscous flux: du - dt 0 == du)
#pragma unroll
      for (int v = IVX; v <= IVZ; ++v) {
        const real* f1 = VF1 + (v - IVX) * f1stride + jt * nf1 + ii;
        real dv = a1 * f1[1] - a1 * f1[0];
        if (has2) {
          const real* f2 = VF2 + (v - IVX) * f2stride + jt * nx1 + ii;
          dv = dv + (a2 * f2[nx1] - a2 * f2[0]);
        }
        if (B.dv3v)  // 3-D: the x3 faces' viscous difference
          dv = dv + static_cast<const real*>(B.dv3v)[(v - IVX) * icells + vci];
        du[v] = du[v] - rdt * vdiv(dv, vol, rvol);
      }
    }
    if (wb) {
      // face-form work + corrected potential-energy work - the cell work
      const int k = ii;
      const real* fm = F1 + IDN * f1stride + jt * nf1;  // fm[k] = face il+k
      auto drho = [&](int kk) -> real {
        real vmd = vdiv(a1 * fm[kk + 1] - a1 * fm[kk], vol, rvol);
        return mdt * vmd;
      };
      // the x1 geometry's constants of interior cell k (slope weights w0,
      // w1, w2 of the corrected PE, g h^2 / 12, g dz above and below the
      // centre), precomputed per block in FP64
      real hi = xt_r(k, 4);
      real lo = xt_r(k, 5);
      real fgw = rdt * vdiv(hi * (a1 * fm[k + 1]) - lo * (a1 * fm[k]), vol, rvol);
      if (nx1 >= 3) {
        int kc = k < 1 ? 1 : (k > nx1 - 2 ? nx1 - 2 : k);
        int k0 = kc - 1;
        real gvar = xt_r(k, 3);
        real sl = xt_r(k, 0) * drho(k0);
        sl += xt_r(k, 1) * drho(k0 + 1);
        sl += xt_r(k, 2) * drho(k0 + 2);
        fgw += gvar * sl;
      }
      const real rho = W[IDN * wstride + wc], vx = W[IVX * wstride + wc];
      real orig = rdt * rho * vx * g * real(1.);
      du[IPR] += fgw - orig;
    }
    if (B.implicit) {
      // the vertical implicit correction follows: hand the explicit
      // tendency to it (interior cell (column, layer) of the VIC scratch)
      double* DU = B.vic;
#pragma unroll
      for (int v = 0; v < NHYDRO; ++v) DU[v * icells + vci] = as_f64(du[v]);
      continue;
    }
#pragma unroll
    for (int v = 0; v < NHYDRO; ++v) {
      const size_t q = v * plane + c;
      uout[q] = w0 * u0[q] + w1 * uin[q] + w2 * du[v];
    }
  }
  if (nclamp && p.counts)
    atomicAdd(&p.counts[bi * kCountSlots + kCountPstar], (unsigned long long)nclamp);
  return true;
}

// the stage of every tile of the batch in ONE persistent launch: a grid of
// (SMs x resident CTAs) walks the tiles of all blocks, uneven blocks
// interleaved so the work per CTA evens out
template <int RK, bool SHOCK>
__global__ void __launch_bounds__(kThreads)
    stage_kernel(const BlockDev* __restrict__ tab, StageParams p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  real* sm = reinterpret_cast<real*>(smem_raw);
  __shared__ uint64_t bar;  // the staging barrier, one phase per bulk tile
  __shared__ int fail;
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncthreads();
  uint32_t phase = 0;
  for (int tile = blockIdx.x; tile < p.ntile; tile += gridDim.x) {
    if (!stage_tile<RK, SHOCK>(tab, p, tile, sm, &bar, phase, &fail)) return;
    __syncthreads();  // the next tile reuses the shared memory
  }
}

// one index of a ghost cell mapped to the interior cell its value comes from
// (src/bc/bc_func.cpp:10-70); flips the sign when a reflecting face maps it
__device__ __forceinline__ int ghost_src(int i, int n, int ng, int lo_kind,
                                         int hi_kind, bool& flip) {
  if (n == 1) return i;
  if (i < ng) {
    if (lo_kind == kBcReflecting) {
      flip = !flip;
      return 2 * ng - 1 - i;
    }
    if (lo_kind == kBcPeriodic) return i + n - 2 * ng;
    if (lo_kind == kBcExtrapolation) return ng;
    return -1;
  }
  if (i >= n - ng) {
    if (hi_kind == kBcReflecting) {
      flip = !flip;
      return 2 * (n - ng) - 1 - i;
    }
    if (hi_kind == kBcPeriodic) return i - (n - 2 * ng);
    if (hi_kind == kBcExtrapolation) return n - ng - 1;
    return -1;
  }
  return i;
}

// the boundary functions of every ghost cell of buf[which], applied as the
// composition of the per-axis maps (equal to applying the faces in the
// order x1, x2, x3 as apply_boundaries does, meshblock_exchange.cpp:214-286)
__global__ void __launch_bounds__(kThreads)
    ghost_kernel(const BlockDev* __restrict__ tab, int which) {
  const BlockDev& B = tab[blockIdx.y];
  const int nc1 = B.nc1, nc2 = B.nc2, nc3 = B.nc3, ng = B.ng;
  const size_t plane = (size_t)nc1 * nc2 * nc3;
  real* q = static_cast<real*>(B.buf[which]);
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < plane;
       c += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(c % nc1);
    const int j = (int)((c / nc1) % nc2);
    const int k = (int)(c / ((size_t)nc1 * nc2));
    bool f1 = false, f2 = false, f3 = false;
    const int si = ghost_src(i, nc1, ng, B.bc[0], B.bc[1], f1);
    const int sj = ghost_src(j, nc2, ng, B.bc[2], B.bc[3], f2);
    const int sk = ghost_src(k, nc3, ng, B.bc[4], B.bc[5], f3);
    if (si == i && sj == j && sk == k) continue;  // interior
    if (si < 0 || sj < 0 || sk < 0) continue;     // no boundary function
    const size_t s = ((size_t)sk * nc2 + sj) * nc1 + si;
#pragma unroll
    for (int v = 0; v < NHYDRO; ++v) {
      real val = q[v * plane + s];
      if ((v == IVX && f1) || (v == IVY && f2) || (v == IVZ && f3))
        val = val * real(-1);
      q[v * plane + c] = val;
    }
    // anomalies: the total copied from x1 row si to row i changes base
    if (B.base && si != i) {
      const double* rb = base_rho(B.base, nc1);
      const double* eb = base_e(B.base, nc1);
      q[IDN * plane + c] += real(rb[si] - rb[i]);
      q[IPR * plane + c] += real(eb[si] - eb[i]);
    }
  }
}

// ---------------------------------------------------------------------------
// passive scalars (ScalarImpl::forward, src/scalar/scalar.cpp:90-211, the
// dry case without the upper bound).  One thread per face of the
// interior cells: the side the stage's mass flux F_m selects (F_m > 0: the
// left state, the plus side of cell f - 1; else the right state, the minus
// side of cell f) is reconstructed by scale-invariant WENO5 for the total
// dry density and each tracer density, floored at 0 (ReconstructImpl::
// forward without a hydro parent, src/recon/reconstruct.cpp:258-262); the
// face ratio r = s_f / rho_f, or the donor cell's where rho_f is not
// positive; the upwind flux F_s = F_m r (riemann.cpp:164-170), zero on the
// reflecting faces (boundary.prescribed), FP64 as the reference keeps it.
// With the flux-covariance row (x2 and x3 faces of blocks with nx1 >= 3) the
// flux adds the tracer row s2 rho D1[u_n] D1[q] (HydroImpl::
// scalar_flux_covariance, src/hydro/hydro_forward.cpp:233-300: q the mean
// of the two sides' ratios, rho and u_n of the hydro's face means, D1 the
// centred x1 difference), and the positivity limiter below follows.
// ---------------------------------------------------------------------------
// the ratio of one side of face q (stride st) of tracer sv
template <typename RHO>
__device__ __forceinline__ real scalar_face_ratio(const real* sv, RHO rho,
                                                  size_t q, size_t st,
                                                  bool left) {
  const size_t c0 = q - (left ? 3 : 2) * st;
  const size_t donor = left ? q - st : q;
  auto face = [&](real f0, real f1, real f2, real f3, real f4) -> real {
    real v = left ? weno5_cp(f0, f1, f2, f3, f4, true)
                  : weno5_cm(f0, f1, f2, f3, f4, true);
    return v < real(0) ? real(0) : v;  // clamp_min: -0 stays
  };
  const real rf = face(rho(c0), rho(c0 + st), rho(c0 + 2 * st),
                       rho(c0 + 3 * st), rho(c0 + 4 * st));
  const real sf = face(sv[c0], sv[c0 + st], sv[c0 + 2 * st], sv[c0 + 3 * st],
                       sv[c0 + 4 * st]);
  return rf > real(0) ? sf / rf : sv[donor] / rho(donor);
}

__global__ void __launch_bounds__(kThreads)
    scalar_flux_kernel(const BlockDev* __restrict__ tab, StageParams p) {
  const BlockDev& B = tab[blockIdx.y];
  const int ns = B.nscalar;
  if (ns == 0) return;
  const int nc1 = B.nc1, nc2 = B.nc2, nc3 = B.nc3, ng = B.ng;
  const bool has2 = nc2 > 1, has3 = nc3 > 1;
  const size_t kst = (size_t)nc1 * nc2, plane = kst * nc3;
  const int nx1 = nc1 - 2 * ng, nx2 = has2 ? nc2 - 2 * ng : 1,
            nx3 = has3 ? nc3 - 2 * ng : 1;
  const int jl = has2 ? ng : 0, kl = has3 ? ng : 0;
  const size_t n1f = (size_t)nx3 * nx2 * (nx1 + 1);
  const size_t n2f = has2 ? (size_t)nx3 * (nx2 + 1) * nx1 : 0;
  const size_t n3f = has3 ? (size_t)(nx3 + 1) * nx2 * nx1 : 0;
  const real* u = static_cast<const real*>(B.buf[p.in]);
  const real* s = static_cast<const real*>(B.sbuf[p.in]);
  const double* rb = B.base ? base_rho(B.base, nc1) : nullptr;
  const real gammad = real(B.gammad);
  const bool scale = p.scale != 0;
  const bool covs = B.flux_cov && nc1 >= 3;
  // the total dry density (the state holds an anomaly under a base)
  auto rho = [&](size_t c) -> real {
    real v = u[IDN * plane + c];
    if (rb) v = v + real(rb[c % nc1]);
    return v;
  };
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
       t < n1f + n2f + n3f; t += (size_t)gridDim.x * blockDim.x) {
    int d, i, j, k;  // the face along d below cell (k, j, i)
    if (t < n1f) {
      d = 0;
      i = ng + (int)(t % (nx1 + 1));
      const size_t r = t / (nx1 + 1);
      j = jl + (int)(r % nx2);
      k = kl + (int)(r / nx2);
    } else if (t < n1f + n2f) {
      const size_t e = t - n1f;
      d = 1;
      i = ng + (int)(e % nx1);
      const size_t r = e / nx1;
      j = ng + (int)(r % (nx2 + 1));
      k = kl + (int)(r / (nx2 + 1));
    } else {
      const size_t e = t - n1f - n2f;
      d = 2;
      i = ng + (int)(e % nx1);
      const size_t r = e / nx1;
      j = jl + (int)(r % nx2);
      k = ng + (int)(r / nx2);
    }
    const size_t q = (size_t)k * kst + (size_t)j * nc1 + i;
    const size_t st = d == 0 ? 1 : (d == 1 ? (size_t)nc1 : kst);
    const int f = d == 0 ? i : (d == 1 ? j : k);
    const int nd = d == 0 ? nc1 : (d == 1 ? nc2 : nc3);
    const bool wall = (f == ng && B.bc[2 * d] == kBcReflecting) ||
                      (f == nd - ng && B.bc[2 * d + 1] == kBcReflecting);
    const double F = B.mflux[d][q];
    const bool left = F > 0.;
    const bool cov = covs && d >= 1;
    // the hydro's face means on the x1 rows i - 1, i, i + 1: the normal
    // velocity, and rho on row i (the hydro's face states, its scheme)
    real un[3] = {real(0), real(0), real(0)}, rhof = real(0);
    if (cov) {
      const int vn = d == 1 ? IVY : IVZ;
      for (int m = -1; m <= 1; ++m) {
        real wd[6], wv[6];
        for (int o = 0; o < 6; ++o) {
          const size_t c = q + m + (o - 3) * st;
          real uc[NHYDRO], w[NHYDRO];
#pragma unroll
          for (int v = 0; v < NHYDRO; ++v) uc[v] = u[v * plane + c];
          if (rb) uc[IDN] = real(rb[c % nc1]) + uc[IDN];
          cons2prim<real>(uc, w, gammad);
          wd[o] = w[IDN];
          wv[o] = w[vn];
        }
        real vl, vr;
        if (p.shock) {
          vl = weno5_cp(wv[0], wv[1], wv[2], wv[3], wv[4], scale);
          vr = weno5_cm(wv[1], wv[2], wv[3], wv[4], wv[5], scale);
        } else {
          vl = cp5_cp(wv[0], wv[1], wv[2], wv[3], wv[4]);
          vr = cp5_cm(wv[1], wv[2], wv[3], wv[4], wv[5]);
        }
        un[m + 1] = real(0.5) * (vl + vr);
        if (m == 0) {
          const real dl = weno5_cp(wd[0], wd[1], wd[2], wd[3], wd[4], scale);
          const real dr = weno5_cm(wd[1], wd[2], wd[3], wd[4], wd[5], scale);
          rhof = real(0.5) * (dl + dr);
        }
      }
    }
    for (int v = 0; v < ns; ++v) {
      const real* sv = s + (size_t)v * plane;
      const real r = scalar_face_ratio(sv, rho, q, st, left);
      double fl = F * (double)r;
      if (cov) {
        real qf[3];
        for (int m = -1; m <= 1; ++m)
          qf[m + 1] = real(0.5) * (scalar_face_ratio(sv, rho, q + m, st, true) * real(1) +
                                   scalar_face_ratio(sv, rho, q + m, st, false) * real(1));
        const real dx1 = real(B.x1v[i + 1] - B.x1v[i - 1]);
        const real s2 = real(B.dx1 * B.dx1 / 12.);
        const real d1u = (un[2] - un[0]) / dx1;
        const real d1q = (qf[2] - qf[0]) / dx1;
        fl = fl + (double)(s2 * rhof * d1u * d1q);
      }
      B.sflux[d][(size_t)v * plane + q] = wall ? 0. : fl;
    }
  }
}

// the positivity limiter of the scalars (PositivityLimiter::apply with the
// scalars' inputs, src/hydro/flux_positivity.cpp:29-268; no energy carry):
// one thread per interior cell and scalar.
//   theta = min(1, s V (1 - 4096 eps) / (dt out)), out the outgoing A F_s
//   over the cell's faces (1 where nothing drains); td the same of the dry
//   density under the mass fluxes; phi = clamp(min of the neighbours'
//   s / rho over each resolved axis / its own, 0, 1) (0 where s / rho is
//   not positive); theta <- theta + phi (min(theta / td, 1) - theta) where
//   0 < td < 1 (flux_positivity_relax)
__global__ void __launch_bounds__(kThreads)
    scalar_theta_kernel(const BlockDev* __restrict__ tab, StageParams p) {
  const BlockDev& B = tab[blockIdx.y];
  const int ns = B.nscalar;
  if (ns == 0 || !(B.flux_cov && B.nc1 >= 3 && (B.nc2 > 1 || B.nc3 > 1))) return;
  const int nc1 = B.nc1, nc2 = B.nc2, nc3 = B.nc3, ng = B.ng;
  const bool has2 = nc2 > 1, has3 = nc3 > 1;
  const size_t kst = (size_t)nc1 * nc2, plane = kst * nc3;
  const int nx1 = nc1 - 2 * ng, nx2 = has2 ? nc2 - 2 * ng : 1,
            nx3 = has3 ? nc3 - 2 * ng : 1;
  const int jl = has2 ? ng : 0, kl = has3 ? ng : 0;
  const double area[3] = {B.dx3 * B.dx2, B.dx3 * B.dx1, B.dx2 * B.dx1};
  const double vol = B.dx3 * (B.dx2 * B.dx1);
  const double dt = p.dt[blockIdx.y];
  const double margin = 4096. * 2.220446049250313e-16;
  const double tiny = 2.2250738585072014e-308;
  const size_t st[3] = {1, (size_t)nc1, kst};
  const bool act[3] = {true, has2, has3};
  const real* u = static_cast<const real*>(B.buf[p.in]);
  const real* s = static_cast<const real*>(B.sbuf[p.in]);
  const double* rb = B.base ? base_rho(B.base, nc1) : nullptr;
  auto rho = [&](size_t c) -> real {
    real v = u[IDN * plane + c];
    if (rb) v = v + real(rb[c % nc1]);
    return v;
  };
  // theta of a channel: densities q (by a functor), face fluxes F[d]
  auto theta_of = [&](size_t c, double qc, const double* const* F) {
    double out = 0.;
    for (int d = 0; d < 3; ++d) {
      if (!act[d]) continue;
      const double up = area[d] * F[d][c + st[d]], dn = area[d] * F[d][c];
      out = out + ((up > 0. ? up : 0.) + (-dn > 0. ? -dn : 0.));
    }
    const double avail = (qc > 0. ? qc : 0.) * vol * (1. - margin);
    const double drain = dt * out;
    if (!(drain > 0.)) return 1.;
    const double t = avail / (drain > tiny ? drain : tiny);
    return t < 1. ? t : 1.;
  };
  const size_t inner = (size_t)nx1 * nx2 * nx3;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
       t < inner * ns; t += (size_t)gridDim.x * blockDim.x) {
    const int v = (int)(t / inner);
    const size_t e = t - (size_t)v * inner;
    const int i = ng + (int)(e % nx1);
    const size_t r = e / nx1;
    const int j = jl + (int)(r % nx2), k = kl + (int)(r / nx2);
    const size_t c = (size_t)k * kst + (size_t)j * nc1 + i;
    const real* sv = s + (size_t)v * plane;
    const double* Fs[3] = {B.sflux[0] + (size_t)v * plane,
                           B.sflux[1] ? B.sflux[1] + (size_t)v * plane : nullptr,
                           B.sflux[2] ? B.sflux[2] + (size_t)v * plane : nullptr};
    const double* Fm[3] = {B.mflux[0], B.mflux[1], B.mflux[2]};
    const double th = theta_of(c, (double)sv[c], Fs);
    const double td = theta_of(c, (double)rho(c), Fm);
    const double qc = (double)(sv[c] / rho(c));
    double low = 0.;
    for (int d = 0; d < 3; ++d) {
      if (!act[d]) continue;
      const double qm = (double)(sv[c - st[d]] / rho(c - st[d]));
      const double qp = (double)(sv[c + st[d]] / rho(c + st[d]));
      const double mm = qm < qp ? qm : qp;
      low = d == 0 ? mm : (mm < low ? mm : low);
    }
    double phi = 0.;
    if (qc > 0.) {
      phi = low / qc;
      phi = phi < 0. ? 0. : (phi > 1. ? 1. : phi);
    }
    double out = th;
    if (td < 1. && td > 0.) {
      const double rr = th / td;
      out = th + phi * ((rr < 1. ? rr : 1.) - th);
    }
    B.stheta[(size_t)v * plane + c] = out;
  }
}

// theta's ghost cells (flux_positivity_sync_theta_: the boundary functions
// of a kScalar field), then each face flux of the interior cells times its
// donor's theta (the lower cell where F_s > 0; flux_positivity_factor)
__global__ void __launch_bounds__(kThreads)
    scalar_theta_ghost_kernel(const BlockDev* __restrict__ tab) {
  const BlockDev& B = tab[blockIdx.y];
  if (B.nscalar == 0 || !(B.flux_cov && B.nc1 >= 3 && (B.nc2 > 1 || B.nc3 > 1)))
    return;
  const int nc1 = B.nc1, nc2 = B.nc2, nc3 = B.nc3, ng = B.ng;
  const size_t plane = (size_t)nc1 * nc2 * nc3;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < plane;
       c += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(c % nc1);
    const int j = (int)((c / nc1) % nc2);
    const int k = (int)(c / ((size_t)nc1 * nc2));
    bool f1 = false, f2 = false, f3 = false;
    const int si = ghost_src(i, nc1, ng, B.bc[0], B.bc[1], f1);
    const int sj = ghost_src(j, nc2, ng, B.bc[2], B.bc[3], f2);
    const int sk = ghost_src(k, nc3, ng, B.bc[4], B.bc[5], f3);
    if (si == i && sj == j && sk == k) continue;  // interior
    for (int v = 0; v < B.nscalar; ++v)
      B.stheta[(size_t)v * plane + c] =
          (si < 0 || sj < 0 || sk < 0)
              ? 1.
              : B.stheta[(size_t)v * plane + ((size_t)sk * nc2 + sj) * nc1 + si];
  }
}

__global__ void __launch_bounds__(kThreads)
    scalar_scale_kernel(const BlockDev* __restrict__ tab) {
  const BlockDev& B = tab[blockIdx.y];
  const int ns = B.nscalar;
  if (ns == 0 || !(B.flux_cov && B.nc1 >= 3 && (B.nc2 > 1 || B.nc3 > 1))) return;
  const int nc1 = B.nc1, nc2 = B.nc2, nc3 = B.nc3, ng = B.ng;
  const bool has2 = nc2 > 1, has3 = nc3 > 1;
  const size_t kst = (size_t)nc1 * nc2, plane = kst * nc3;
  const int nx1 = nc1 - 2 * ng, nx2 = has2 ? nc2 - 2 * ng : 1,
            nx3 = has3 ? nc3 - 2 * ng : 1;
  const int jl = has2 ? ng : 0, kl = has3 ? ng : 0;
  const size_t n1f = (size_t)nx3 * nx2 * (nx1 + 1);
  const size_t n2f = has2 ? (size_t)nx3 * (nx2 + 1) * nx1 : 0;
  const size_t n3f = has3 ? (size_t)(nx3 + 1) * nx2 * nx1 : 0;
  const size_t nf = n1f + n2f + n3f;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < nf * ns;
       t += (size_t)gridDim.x * blockDim.x) {
    const int v = (int)(t / nf);
    const size_t tf = t - (size_t)v * nf;
    int d, i, j, k;
    if (tf < n1f) {
      d = 0;
      i = ng + (int)(tf % (nx1 + 1));
      const size_t r = tf / (nx1 + 1);
      j = jl + (int)(r % nx2);
      k = kl + (int)(r / nx2);
    } else if (tf < n1f + n2f) {
      const size_t e = tf - n1f;
      d = 1;
      i = ng + (int)(e % nx1);
      const size_t r = e / nx1;
      j = ng + (int)(r % (nx2 + 1));
      k = kl + (int)(r / (nx2 + 1));
    } else {
      const size_t e = tf - n1f - n2f;
      d = 2;
      i = ng + (int)(e % nx1);
      const size_t r = e / nx1;
      j = jl + (int)(r % nx2);
      k = ng + (int)(r / nx2);
    }
    const size_t q = (size_t)k * kst + (size_t)j * nc1 + i;
    const size_t st = d == 0 ? 1 : (d == 1 ? (size_t)nc1 : kst);
    double* F = B.sflux[d] + (size_t)v * plane + q;
    const double* th = B.stheta + (size_t)v * plane;
    const double fac = *F > 0. ? th[q - st] : th[q];
    *F = *F * fac;
  }
}

// ds = -dt div F_s on the interior cells (the area-weighted divergence, in
// the hydro's order), then the stage's combine s_out = w0 s0 + w1 s + w2 ds
__global__ void __launch_bounds__(kThreads)
    scalar_update_kernel(const BlockDev* __restrict__ tab, StageParams p) {
  const BlockDev& B = tab[blockIdx.y];
  const int ns = B.nscalar;
  if (ns == 0) return;
  const int nc1 = B.nc1, nc2 = B.nc2, nc3 = B.nc3, ng = B.ng;
  const bool has2 = nc2 > 1, has3 = nc3 > 1;
  const size_t kst = (size_t)nc1 * nc2, plane = kst * nc3;
  const int nx1 = nc1 - 2 * ng, nx2 = has2 ? nc2 - 2 * ng : 1,
            nx3 = has3 ? nc3 - 2 * ng : 1;
  const int jl = has2 ? ng : 0, kl = has3 ? ng : 0;
  const double a1 = B.dx3 * B.dx2, a2 = B.dx3 * B.dx1, a3 = B.dx2 * B.dx1;
  const double vol = B.dx3 * (B.dx2 * B.dx1);
  const double mdt = -p.dt[blockIdx.y];
  const real* s0 = static_cast<const real*>(B.sbuf[p.u0]);
  const real* s = static_cast<const real*>(B.sbuf[p.in]);
  real* so = static_cast<real*>(B.sbuf[p.out]);
  const size_t inner = (size_t)nx1 * nx2 * nx3;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
       t < inner * ns; t += (size_t)gridDim.x * blockDim.x) {
    const int v = (int)(t / inner);
    const size_t e = t - (size_t)v * inner;
    const int i = ng + (int)(e % nx1);
    const size_t r = e / nx1;
    const int j = jl + (int)(r % nx2), k = kl + (int)(r / nx2);
    const size_t q = (size_t)v * plane + (size_t)k * kst + (size_t)j * nc1 + i;
    const double* F1 = B.sflux[0];
    double dv = a1 * F1[q + 1] - a1 * F1[q];
    if (has2) {
      const double* F2 = B.sflux[1];
      dv = dv + (a2 * F2[q + nc1] - a2 * F2[q]);
    }
    if (has3) {
      const double* F3 = B.sflux[2];
      dv = dv + (a3 * F3[q + kst] - a3 * F3[q]);
    }
    const double ds = mdt * (dv / vol);
    if (B.implicit)
      B.sds[q] = ds;  // the solve's transfer and the update follow
    else
      so[q] = real(p.w0 * (double)s0[q] + p.w1 * (double)s[q] + p.w2 * ds);
  }
}

// the scalars' ghost cells of sbuf[which]: the boundary functions of a
// kScalar field (bc_func.cpp:10-70), the state's maps without sign flips
__global__ void __launch_bounds__(kThreads)
    scalar_ghost_kernel(const BlockDev* __restrict__ tab, int which) {
  const BlockDev& B = tab[blockIdx.y];
  if (B.nscalar == 0) return;
  const int nc1 = B.nc1, nc2 = B.nc2, nc3 = B.nc3, ng = B.ng;
  const size_t plane = (size_t)nc1 * nc2 * nc3;
  real* q = static_cast<real*>(B.sbuf[which]);
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < plane;
       c += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(c % nc1);
    const int j = (int)((c / nc1) % nc2);
    const int k = (int)(c / ((size_t)nc1 * nc2));
    bool f1 = false, f2 = false, f3 = false;
    const int si = ghost_src(i, nc1, ng, B.bc[0], B.bc[1], f1);
    const int sj = ghost_src(j, nc2, ng, B.bc[2], B.bc[3], f2);
    const int sk = ghost_src(k, nc3, ng, B.bc[4], B.bc[5], f3);
    if (si == i && sj == j && sk == k) continue;  // interior
    if (si < 0 || sj < 0 || sk < 0) continue;     // no boundary function
    const size_t src = ((size_t)sk * nc2 + sj) * nc1 + si;
    for (int v = 0; v < B.nscalar; ++v)
      q[(size_t)v * plane + c] = q[(size_t)v * plane + src];
  }
}

// the x3 faces of 3-D blocks (CoordinateImpl::divergence's x3 term,
// src/coord/coordinate.cpp:650-656): one thread per (x1 cell, x2 row, chunk
// of kX3Chunk x3 cells) walks the chunk's faces with a sliding window of six
// primitives in registers, solves each face once and stores a3 (F3[k+1] -
// F3[k]) of each cell, which the stage kernel adds to its divergence after
// the x1 and x2 differences, the reference's order.  With a hydrostatic base the
// pressure is the anomaly about the cell row's base, as on x2 faces; the
// covariance row (src/hydro/hydro_forward.cpp:58-231 with dim 3, added to
// the face flux before the walls, :800-826) is added to the energy row; a
// reflecting x3 wall zeroes the mass and energy rows of its face.
constexpr int kX3Chunk = 16;

// 3-D viscosity's prep (DiffusionImpl::cartesian_fluxes, src/forcing/
// diffusion.cpp:553-683): on the interior extended by one cell in each
// direction, the velocity divergence (the x1, x2, x3 centred derivatives
// summed in that order) and the centred derivatives dv1/dx3, dv2/dx3 (the
// x1 and x2 faces' shear along x3) and dv3/dx1, dv3/dx2 (the x3 faces'),
// one thread per cell, into the block's five visc3 planes
__global__ void __launch_bounds__(kThreads)
    visc3_kernel(const BlockDev* __restrict__ tab, StageParams p) {
  const BlockDev& B = tab[blockIdx.y];
  if (B.nc3 == 1 || !(B.nu_iso > 0.)) return;
  const int nc1 = B.nc1, nc2 = B.nc2, nc3 = B.nc3, ng = B.ng;
  const bool has2 = nc2 > 1;
  const size_t kst = (size_t)nc1 * nc2, plane = kst * nc3;
  const int e1 = nc1 - 2 * ng + 2, e2 = has2 ? nc2 - 2 * ng + 2 : 1,
            e3 = nc3 - 2 * ng + 2;
  const int o2 = has2 ? ng - 1 : 0;
  const real* u = static_cast<const real*>(B.buf[p.in]);
  const real gammad = real(B.gammad);
  const double* rb = B.base ? base_rho(B.base, nc1) : nullptr;
  real* V = static_cast<real*>(B.visc3);
  const real d2x1 = real(2.) * real(B.dx1), d2x2 = real(2.) * real(B.dx2),
             d2x3 = real(2.) * real(B.dx3);
  const real r1 = real(1.) / d2x1, r2 = real(1.) / d2x2, r3 = real(1.) / d2x3;
  auto vel = [&](size_t c, int v) -> real {
    real uc[NHYDRO], w[NHYDRO];
#pragma unroll
    for (int q = 0; q < NHYDRO; ++q) uc[q] = u[q * plane + c];
    if (rb) uc[IDN] = real(rb[c % nc1]) + uc[IDN];
    cons2prim<real>(uc, w, gammad);
    return w[v];
  };
  const size_t total = (size_t)e1 * e2 * e3;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const int i = ng - 1 + (int)(e % e1);
    const int j = o2 + (int)((e / e1) % e2);
    const int k = ng - 1 + (int)(e / ((size_t)e1 * e2));
    const size_t c = (size_t)k * kst + (size_t)j * nc1 + i;
    real dv = real(0);
    dv += vdiv(vel(c + 1, IVX) - vel(c - 1, IVX), d2x1, r1);
    if (has2) dv += vdiv(vel(c + nc1, IVY) - vel(c - nc1, IVY), d2x2, r2);
    dv += vdiv(vel(c + kst, IVZ) - vel(c - kst, IVZ), d2x3, r3);
    V[c] = dv;
    V[plane + c] = vdiv(vel(c + kst, IVX) - vel(c - kst, IVX), d2x3, r3);
    V[2 * plane + c] = has2 ? vdiv(vel(c + kst, IVY) - vel(c - kst, IVY), d2x3, r3)
                            : real(0);
    V[3 * plane + c] = vdiv(vel(c + 1, IVZ) - vel(c - 1, IVZ), d2x1, r1);
    V[4 * plane + c] = has2 ? vdiv(vel(c + nc1, IVZ) - vel(c - nc1, IVZ), d2x2, r2)
                            : real(0);
  }
}

template <int RK, bool SHOCK>
__global__ void __launch_bounds__(kThreads)
    x3_kernel(const BlockDev* __restrict__ tab, StageParams p) {
  const BlockDev& B = tab[blockIdx.y];
  if (B.nc3 == 1) return;
  const int nc1 = B.nc1, nc2 = B.nc2, nc3 = B.nc3, ng = B.ng;
  const int nx1 = nc1 - 2 * ng, nx2 = nc2 > 1 ? nc2 - 2 * ng : 1,
            nx3 = nc3 - 2 * ng;
  const int o2 = nc2 > 1 ? ng : 0;
  const int nch = (nx3 + kX3Chunk - 1) / kX3Chunk;
  const size_t plane = (size_t)nc1 * nc2 * nc3, kst = (size_t)nc1 * nc2;
  const real* __restrict__ uin = static_cast<const real*>(B.buf[p.in]);
  const real gammad = real(B.gammad);
  const bool scale = p.scale != 0;
  const double* rb = B.base ? base_rho(B.base, nc1) : nullptr;
  const double* pbc = B.base ? base_p(B.base, nc1) : nullptr;
  const real a3 = real(B.dx2 * B.dx1);
  const bool wlo = B.bc[4] == kBcReflecting, whi = B.bc[5] == kBcReflecting;
  // the covariance row of the x3 faces (_flux_covariance, dim 3) needs each
  // face's mean state on the x1 rows either side: a warp then covers 32
  // consecutive x1 rows of one (x2, chunk) line -- 30 it owns and a row
  // either side (an x1 ghost row at the column's ends) -- and trades the
  // face means by shuffles; every lane of a warp runs the same faces
  const bool cov = B.flux_cov && nc1 >= 3;
  const bool visc = B.nu_iso > 0.;
  const size_t vplane = plane;  // one visc3 plane
  const int nw = (nx1 + 29) / 30;  // warps per (x2, chunk) line
  const size_t total = cov ? (size_t)32 * nw * nx2 * nch
                           : (size_t)nx1 * nx2 * nch;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    int i, j, ch;
    bool own = true;
    if (cov) {
      const int lane = (int)(e & 31);
      const size_t wdx = e >> 5;
      const int row = ng - 1 + 30 * (int)(wdx % nw) + lane;
      j = o2 + (int)((wdx / nw) % nx2);
      ch = (int)(wdx / ((size_t)nw * nx2));
      own = lane >= 1 && lane <= 30 && row < ng + nx1;
      i = row < ng + nx1 ? row : ng + nx1;  // past the top ghost row: a copy
    } else {
      i = ng + (int)(e % nx1);
      j = o2 + (int)((e / nx1) % nx2);
      ch = (int)(e / ((size_t)nx1 * nx2));
    }
    const int k0 = ng + ch * kX3Chunk;
    const int k1 = min(k0 + kX3Chunk, ng + nx3);  // cells k0..k1-1
    const size_t col = (size_t)j * nc1 + i;
    const real pb = pbc ? real(pbc[i]) : real(0);
    auto load = [&](int k, real* w) {
      real uc[NHYDRO];
#pragma unroll
      for (int v = 0; v < NHYDRO; ++v) uc[v] = uin[v * plane + k * kst + col];
      if (rb) uc[IDN] = real(rb[i]) + uc[IDN];
      cons2prim<real>(uc, w, gammad);
    };
    // window: cells f-3 .. f+2 of face f
    real W[6][NHYDRO];
#pragma unroll
    for (int m = 0; m < 5; ++m) load(k0 - 3 + m, W[m]);
    real fprev[NHYDRO], vprev[3] = {real(0), real(0), real(0)};
    for (int f = k0; f <= k1; ++f) {
      load(f + 2, W[5]);
      real wl[NHYDRO], wr[NHYDRO], flx[NHYDRO];
#pragma unroll
      for (int v = 0; v < NHYDRO; ++v) {
        if (SHOCK || v == IDN) {
          wl[v] = weno5_cp(W[0][v], W[1][v], W[2][v], W[3][v], W[4][v], scale);
          wr[v] = weno5_cm(W[1][v], W[2][v], W[3][v], W[4][v], W[5][v], scale);
        } else {
          wl[v] = cp5_cp(W[0][v], W[1][v], W[2][v], W[3][v], W[4][v]);
          wr[v] = cp5_cm(W[1][v], W[2][v], W[3][v], W[4][v], W[5][v]);
        }
      }
      real dcov = real(0);
      if (cov) {
        // the face mean's rho, h = (p / (gamma - 1) + p) / rho (p the
        // total) and u_n; the covariance s2 rho D1[h] D1[u_n] of the owned
        // rows from their neighbours' (the x2 row's operations)
        real wb_[NHYDRO];
#pragma unroll
        for (int v = 0; v < NHYDRO; ++v) wb_[v] = real(0.5) * (wl[v] + wr[v]);
        real pbar = wb_[IPR];
        if (pbc) pbar = real(pbc[i]) + pbar;
        const real enth = pbar / (gammad - real(1)) + pbar;
        const real hh = enth / wb_[IDN], un = wb_[IVZ];
        const unsigned full = 0xffffffffu;
        const real hm = __shfl_up_sync(full, hh, 1), hp = __shfl_down_sync(full, hh, 1);
        const real um = __shfl_up_sync(full, un, 1), up = __shfl_down_sync(full, un, 1);
        if (own) {
          const real dx1 = real(B.x1v[i + 1] - B.x1v[i - 1]);
          const real s2 = real(B.dx1 * B.dx1 / 12.);
          const real s2rho = s2 * wb_[IDN];
          const real rdx1 = real(1.) / dx1;
          const real d1h = vdiv(hp - hm, dx1, rdx1);
          const real dun = vdiv(up - um, dx1, rdx1);
          dcov = s2rho * d1h * dun;
        }
      }
      if (pbc)
        lmars_flux_anom<real>(wl, wr, gammad, 3, pb, flx);
      else {
        // a chunk owns its faces but the top one (the next chunk's), except
        // the block's last face
        unsigned c = 0;
        riemann<RK>(wl, wr, gammad, 3, flx, c);
        if (c && own && (f < k1 || k1 == ng + nx3) && p.counts)
          atomicAdd(&p.counts[blockIdx.y * kCountSlots + kCountPstar], 1ull);
      }
      if (cov) flx[IPR] += dcov;
      if ((f == ng && wlo) || (f == ng + nx3 && whi))
        flx[IDN] = flx[IPR] = real(0);
      if (!own) {  // a halo lane: its row's face means only
#pragma unroll
        for (int m = 0; m < 5; ++m)
#pragma unroll
          for (int v = 0; v < NHYDRO; ++v) W[m][v] = W[m + 1][v];
        continue;
      }
      // viscosity: the x3 face's viscous fluxes between cells f - 1
      // (W[2]) and f (W[3]); the energy row joins the total (post_fluxes,
      // then the walls again), the momentum rows their own difference
      real vfl[3] = {real(0), real(0), real(0)};
      if (visc) {
        const size_t c = (size_t)f * kst + col, cm = c - kst;
        const real* VP = static_cast<const real*>(B.visc3);
        const real nu = real(B.nu_iso);
        const real dx3 = real(B.dx3), rdx3 = real(1.) / dx3;
        const real rf = real(0.5) * (W[3][IDN] + W[2][IDN]);
        const real divf = real(0.5) * (VP[c] + VP[cm]);
        real e = real(0);
#pragma unroll
        for (int ivar = 0; ivar < 3; ++ivar) {
          const int v = IVX + ivar;
          real stress = vdiv(W[3][v] - W[2][v], dx3, rdx3);
          if (ivar == 2) {
            stress = real(2.) * stress - real(2. / 3.) * divf;
          } else if (ivar == 0) {
            stress += real(0.5) * (VP[3 * vplane + c] + VP[3 * vplane + cm]);
          } else if (nc2 > 1) {
            stress += real(0.5) * (VP[4 * vplane + c] + VP[4 * vplane + cm]);
          }
          const real mf = -nu * rf * stress;
          vfl[ivar] = mf;
          e += real(0.5) * (W[3][v] + W[2][v]) * mf;
        }
        flx[IPR] += e;
        if ((f == ng && wlo) || (f == ng + nx3 && whi))
          flx[IDN] = flx[IPR] = real(0);
      }
      // passive scalars ride on the mass row (the step field's owner rule)
      if (B.nscalar > 0 && (f < k1 || k1 == ng + nx3))
        B.mflux[2][(size_t)f * kst + col] = as_f64(flx[IDN]);
      // the x3 step field; a chunk owns its faces but the top one, which
      // the next chunk owns, except the block's last face
      if (B.step[2] && (f < k1 || k1 == ng + nx3)) {
        const double w2dt = p.w2 * p.dt[blockIdx.y];
        double* S3 = B.step[2] + (size_t)f * kst + col;
#pragma unroll
        for (int v = 0; v < NHYDRO; ++v) {
          double t = as_f64(flx[v]);
          if (pbc && v == IVZ) t = t + pbc[i];
          step_set(S3 + v * plane, t, p.w1, w2dt, p.first != 0);
        }
      }
      if (f > k0) {
        // cell f - 1 between faces f - 1 and f
        const int k = f - 1;
        real* DV3 = static_cast<real*>(B.dv3);
        const size_t cells = (size_t)nx1 * nx2 * nx3;
        const size_t vc = ((size_t)(k - ng) * nx2 + (j - o2)) * nx1 + (i - ng);
#pragma unroll
        for (int v = 0; v < NHYDRO; ++v)
          DV3[v * cells + vc] = a3 * flx[v] - a3 * fprev[v];
        if (visc) {
          real* DVV = static_cast<real*>(B.dv3v);
#pragma unroll
          for (int q = 0; q < 3; ++q)
            DVV[q * cells + vc] = a3 * vfl[q] - a3 * vprev[q];
        }
      }
#pragma unroll
      for (int v = 0; v < NHYDRO; ++v) fprev[v] = flx[v];
#pragma unroll
      for (int q = 0; q < 3; ++q) vprev[q] = vfl[q];
#pragma unroll
      for (int m = 0; m < 5; ++m)
#pragma unroll
        for (int v = 0; v < NHYDRO; ++v) W[m][v] = W[m + 1][v];
    }
  }
}

// U -> W of every cell of buf[which] into out (per block, laid out like buf)
__global__ void __launch_bounds__(kThreads)
    prim_kernel(const BlockDev* __restrict__ tab, int which, void* const* out) {
  const BlockDev& B = tab[blockIdx.y];
  const size_t plane = (size_t)B.nc1 * B.nc2 * B.nc3;
  const real* u = static_cast<const real*>(B.buf[which]);
  real* w = static_cast<real*>(out[blockIdx.y]);
  const real gammad = real(B.gammad);
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < plane;
       c += (size_t)gridDim.x * blockDim.x) {
    real uc[NHYDRO], wc[NHYDRO];
#pragma unroll
    for (int v = 0; v < NHYDRO; ++v) uc[v] = u[v * plane + c];
    if (B.base) uc[IDN] = real(base_rho(B.base, B.nc1)[c % B.nc1]) + uc[IDN];
    cons2prim<real>(uc, wc, gammad);
    if (B.base) wc[IPR] = real(base_p(B.base, B.nc1)[c % B.nc1]) + wc[IPR];
#pragma unroll
    for (int v = 0; v < NHYDRO; ++v) w[v * plane + c] = wc[v];
  }
}

// ideal-gas W->U of one cell, src/eos/ideal_gas.cpp:53-70 (the metric
// lowering is the identity in Cartesian), in FP64
__device__ __forceinline__ void prim2cons64(const double* w, double* u,
                                            double gammad) {
  double rho = w[IDN];
  double m1 = w[IVX] * rho, m2 = w[IVY] * rho, m3 = w[IVZ] * rho;
  u[IDN] = rho;
  u[IVX] = m1;
  u[IVY] = m2;
  u[IVZ] = m3;
  double ke = 0.5 * (w[IVX] * m1 + w[IVY] * m2 + w[IVZ] * m3);
  u[IPR] = w[IPR] / (gammad - 1) + ke;
}

// initialize (src/mesh/meshblock.cpp:306-420): boundary functions on the
// FP64 primitives, W->U, boundary functions on U -- one pass, since the
// boundary maps are copies with sign flips that commute with W->U
__global__ void __launch_bounds__(kThreads)
    init_kernel(const BlockDev* __restrict__ tab, int which,
                double* const* win) {
  const BlockDev& B = tab[blockIdx.y];
  const int nc1 = B.nc1, nc2 = B.nc2, nc3 = B.nc3, ng = B.ng;
  const size_t plane = (size_t)nc1 * nc2 * nc3;
  double* w = win[blockIdx.y];
  real* q = static_cast<real*>(B.buf[which]);
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < plane;
       c += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(c % nc1);
    const int j = (int)((c / nc1) % nc2);
    const int k = (int)(c / ((size_t)nc1 * nc2));
    bool f1 = false, f2 = false, f3 = false;
    int si = ghost_src(i, nc1, ng, B.bc[0], B.bc[1], f1);
    int sj = ghost_src(j, nc2, ng, B.bc[2], B.bc[3], f2);
    int sk = ghost_src(k, nc3, ng, B.bc[4], B.bc[5], f3);
    if (si < 0) si = i, f1 = false;
    if (sj < 0) sj = j, f2 = false;
    if (sk < 0) sk = k, f3 = false;
    const size_t s = ((size_t)sk * nc2 + sj) * nc1 + si;
    double wc[NHYDRO], uc[NHYDRO];
#pragma unroll
    for (int v = 0; v < NHYDRO; ++v) wc[v] = w[v * plane + s];
    if (f1) wc[IVX] = wc[IVX] * -1.;
    if (f2) wc[IVY] = wc[IVY] * -1.;
    if (f3) wc[IVZ] = wc[IVZ] * -1.;
    // the primitives' own ghosts, as apply_boundaries(hydro_w) leaves them
    // (a ghost is never the source of another cell, so this cannot race)
    if (s != c) {
#pragma unroll
      for (int v = 0; v < NHYDRO; ++v) w[v * plane + c] = wc[v];
    }
    prim2cons64(wc, uc, B.gammad);
    if (B.base) {  // the anomaly about the base, formed in FP64
      uc[IDN] = uc[IDN] - base_rho(B.base, nc1)[i];
      uc[IPR] = uc[IPR] - base_e(B.base, nc1)[i];
    }
#pragma unroll
    for (int v = 0; v < NHYDRO; ++v) q[v * plane + c] = real(uc[v]);
  }
}

__device__ __forceinline__ double warp_min(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = fmin(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}
__device__ __forceinline__ int warp_or(int x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x |= __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// per-block reductions over the interior cells of buf[which]:
//   red[4 b + 0] <- min dx_d / (|v_d| + c)   (HydroImpl::max_time_step)
//   red[4 b + 1] <- min rho, red[4 b + 2] <- min p, (as ordered bit patterns)
//   flag[b] |= 1 if any interior value is NaN
__global__ void __launch_bounds__(kThreads)
    reduce_kernel(const BlockDev* __restrict__ tab, int which,
                  unsigned long long* red, int* flag) {
  const int b = blockIdx.y;
  const BlockDev& B = tab[b];
  const int nc1 = B.nc1, nc2 = B.nc2, nc3 = B.nc3, ng = B.ng;
  const int nx1 = nc1 > 1 ? nc1 - 2 * ng : 1, nx2 = nc2 > 1 ? nc2 - 2 * ng : 1,
            nx3 = nc3 > 1 ? nc3 - 2 * ng : 1;
  const int o1 = nc1 > 1 ? ng : 0, o2 = nc2 > 1 ? ng : 0, o3 = nc3 > 1 ? ng : 0;
  const size_t plane = (size_t)nc1 * nc2 * nc3;
  const size_t ncell = (size_t)nx1 * nx2 * nx3;
  const real* u = static_cast<const real*>(B.buf[which]);
  const real gammad = real(B.gammad);
  double dtm = INFINITY, rmin = INFINITY, pmin = INFINITY;
  int nan = 0;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < ncell;
       e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % nx1) + o1;
    const int j = (int)((e / nx1) % nx2) + o2;
    const int k = (int)(e / ((size_t)nx1 * nx2)) + o3;
    const size_t c = ((size_t)k * nc2 + j) * nc1 + i;
    real uc[NHYDRO], w[NHYDRO];
#pragma unroll
    for (int v = 0; v < NHYDRO; ++v) uc[v] = u[v * plane + c];
    if (B.base) uc[IDN] = real(base_rho(B.base, nc1)[i]) + uc[IDN];
    cons2prim<real>(uc, w, gammad);
    if (B.base) w[IPR] = real(base_p(B.base, nc1)[i]) + w[IPR];
    const real cs = sqrt(gammad * w[IPR] / w[IDN]);
    // an implicit x1 (scheme bit 0, more than one column) keeps only the
    // advective bound dx1 / (|v1| cfl / advection_cfl) (hydro.cpp:327-340)
    if (nc1 > 1 && (B.implicit & 1) && !(nc2 == 1 && nc3 == 1))
      dtm = fmin(dtm, (double)(real(B.dx1) / (fabs(w[IVX]) * real(B.cfl / 1.0))));
    else if (nc1 > 1)
      dtm = fmin(dtm, (double)(real(B.dx1) / (fabs(w[IVX]) + cs)));
    if (nc2 > 1) dtm = fmin(dtm, (double)(real(B.dx2) / (fabs(w[IVY]) + cs)));
    if (nc3 > 1) dtm = fmin(dtm, (double)(real(B.dx3) / (fabs(w[IVZ]) + cs)));
    rmin = fmin(rmin, (double)w[IDN]);
    pmin = fmin(pmin, (double)w[IPR]);
#pragma unroll
    for (int v = 0; v < NHYDRO; ++v) nan |= isnan(w[v]) ? 1 : 0;
    nan |= isnan(cs) ? 1 : 0;
  }
  __shared__ double s_dt[kThreads / 32], s_r[kThreads / 32], s_p[kThreads / 32];
  __shared__ int s_n[kThreads / 32];
  dtm = warp_min(dtm);
  rmin = warp_min(rmin);
  pmin = warp_min(pmin);
  nan = warp_or(nan);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    s_dt[wid] = dtm;
    s_r[wid] = rmin;
    s_p[wid] = pmin;
    s_n[wid] = nan;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 1; q < (int)(blockDim.x >> 5); ++q) {
      dtm = fmin(dtm, s_dt[q]);
      rmin = fmin(rmin, s_r[q]);
      pmin = fmin(pmin, s_p[q]);
      nan |= s_n[q];
    }
    // order-preserving keys of doubles for an unsigned atomicMin
    auto key = [](double x) {
      unsigned long long k = __double_as_longlong(x);
      return (k >> 63) ? ~k : (k | 0x8000000000000000ull);
    };
    atomicMin(&red[4 * b + 0], key(fmin(dtm, B.dt_src)));
    atomicMin(&red[4 * b + 1], key(rmin));
    atomicMin(&red[4 * b + 2], key(pmin));
    if (nan) atomicOr(&flag[b], 1);
  }
}

#include "sg_vic.cuh"
#include "sg_psolve.cuh"

// an implicit block's scalars after its solve, one warp per column and
// scalar (MeshBlockImpl::stage_advance, src/mesh/meshblock_advance.cpp:
// 216-233): each x1 face's transfer q carries the donor's ratio r = s / rho
// of the stage input (the cell below where q > 0), P = r q.  The donor cap
// (donor_cap_cpu, src/implicit/implicit_dispatch.cpp:54-70) is tested on
// every interior face at once: P above held below + the face below's P, or
// under -held above, held = max(s + ds, 0) V; only a column where a face
// binds walks from the bottom capping each face to [-held above, what the
// cell below holds plus what it received].  A column with no binding face
// is left as it is, as the reference's walk leaves it.  Then
// ds += (P - P_above) / V and the stage's combine, coalesced over the
// column.  P is kept in the x1 face-flux rows, which the update has read
constexpr int kVicScalarWarps = 4;

__global__ void __launch_bounds__(32 * kVicScalarWarps)
    scalar_vic_kernel(const BlockDev* __restrict__ tab, StageParams p) {
  const BlockDev& B = tab[blockIdx.y];
  const int ns = B.nscalar;
  if (ns == 0 || !B.implicit) return;
  const int nc1 = B.nc1, ng = B.ng, n = nc1 - 2 * ng;
  const size_t plane = (size_t)nc1 * B.nc2 * B.nc3;
  const size_t ncol = (size_t)(B.nc2 > 1 ? B.nc2 - 2 * ng : 1) *
                      (B.nc3 > 1 ? B.nc3 - 2 * ng : 1);
  const int lane = threadIdx.x & 31;
  const size_t task = (size_t)blockIdx.x * kVicScalarWarps + (threadIdx.x >> 5);
  if (task >= ncol * ns) return;  // the whole warp
  const int v = (int)(task / ncol);
  const size_t col = task - (size_t)v * ncol;
  const size_t row = vic_row(B, col) * nc1;
  const real* s = static_cast<const real*>(B.sbuf[p.in]) + v * plane + row;
  const real* s0 = static_cast<const real*>(B.sbuf[p.u0]) + v * plane + row;
  real* so = static_cast<real*>(B.sbuf[p.out]) + v * plane + row;
  const real* u = static_cast<const real*>(B.buf[p.in]) + IDN * plane + row;
  const double* rb = B.base ? base_rho(B.base, nc1) : nullptr;
  const double* ds = B.sds + v * plane + row;
  const double* q = B.vicq + row;
  double* P = B.sflux[0] + v * plane + row;
  const double vol = B.dx3 * (B.dx2 * B.dx1);
  const int il = ng, iu = ng + n - 1;
  auto ratio = [&](int i) -> double {
    real rho = u[i];
    if (rb) rho = rho + real(rb[i]);
    return (double)(s[i] / rho);
  };
  auto held = [&](int i) -> double {
    const double h = (double)s[i] + ds[i];
    return (h < 0. ? 0. : h) * vol;
  };
  for (int f = il + lane; f <= iu + 1; f += 32) {
    const double M = q[f];
    P[f] = (M > 0. ? ratio(f - 1) : ratio(f)) * M;
  }
  __syncwarp();
  bool bind = false;
  for (int f = il + 1 + lane; f <= iu; f += 32) {
    const double cap = held(f - 1) + (f - 1 > il ? P[f - 1] : 0.);
    bind = bind || P[f] > cap || P[f] < -held(f);
  }
  if (__any_sync(0xffffffffu, bind)) {
    if (lane == 0) {
      double avail = held(il);
      for (int f = il + 1; f <= iu; ++f) {
        const double up = held(f);
        double Q = P[f];
        if (Q > avail) Q = avail;
        if (Q < -up) Q = -up;
        P[f] = Q;
        avail = up + Q;
      }
    }
    __syncwarp();
  }
  for (int i = il + lane; i <= iu; i += 32) {
    const double d = ds[i] + (P[i] - P[i + 1]) / vol;
    so[i] = real(p.w0 * (double)s0[i] + p.w1 * (double)s[i] + p.w2 * d);
  }
}


// ---------------------------------------------------------------------------
// the budget sums (BudgetConsumer::totals and ::boundary,
// src/diagnostics/budget.cpp:68-155): one CTA per block, each thread sums a
// fixed stride of the cells (or faces), then a fixed-order tree, so the
// sums are the same on every run and in a captured graph
// ---------------------------------------------------------------------------
constexpr int kBudgetThreads = 512;

__device__ void budget_reduce(double* acc, double* out, bool accumulate) {
  __shared__ double sh[NHYDRO][kBudgetThreads];
  const int t = threadIdx.x;
#pragma unroll
  for (int v = 0; v < NHYDRO; ++v) sh[v][t] = acc[v];
  __syncthreads();
  for (int s = kBudgetThreads / 2; s > 0; s >>= 1) {
    if (t < s) {
#pragma unroll
      for (int v = 0; v < NHYDRO; ++v) sh[v][t] = sh[v][t] + sh[v][t + s];
    }
    __syncthreads();
  }
  if (t < NHYDRO) out[t] = accumulate ? out[t] + sh[t][0] : sh[t][0];
}

// sum over the interior of the total u (the base added back) times the
// cell volume, per row
__global__ void __launch_bounds__(kBudgetThreads)
    budget_totals_kernel(const BlockDev* __restrict__ tab, int which,
                         double* out) {
  const BlockDev& B = tab[blockIdx.x];
  const int nc1 = B.nc1, nc2 = B.nc2, nc3 = B.nc3, ng = B.ng;
  const int nx1 = nc1 - 2 * ng, nx2 = nc2 > 1 ? nc2 - 2 * ng : 1,
            nx3 = nc3 > 1 ? nc3 - 2 * ng : 1;
  const int o2 = nc2 > 1 ? ng : 0, o3 = nc3 > 1 ? ng : 0;
  const size_t plane = (size_t)nc1 * nc2 * nc3;
  const real* u = static_cast<const real*>(B.buf[which]);
  const double* rb = B.base ? base_rho(B.base, nc1) : nullptr;
  const double* eb = B.base ? base_e(B.base, nc1) : nullptr;
  const double vol = B.dx3 * (B.dx2 * B.dx1);
  const size_t n = (size_t)nx1 * nx2 * nx3;
  double acc[NHYDRO] = {0., 0., 0., 0., 0.};
  for (size_t e = threadIdx.x; e < n; e += kBudgetThreads) {
    const int i = ng + (int)(e % nx1);
    const size_t jk = e / nx1;
    const int j = o2 + (int)(jk % nx2), k = o3 + (int)(jk / nx2);
    const size_t c = ((size_t)k * nc2 + j) * nc1 + i;
#pragma unroll
    for (int v = 0; v < NHYDRO; ++v) {
      double x = (double)u[v * plane + c];
      if (rb && v == IDN) x = x + rb[i];
      if (eb && v == IPR) x = x + eb[i];
      acc[v] += x * vol;
    }
  }
  budget_reduce(acc, out + NHYDRO * blockIdx.x, false);
}

// the outward transfer of the step fields through the boundary faces: on
// each boundary face of the interior cells, sign A_f S_d (sign -1 on the
// lower, +1 on the upper face of direction d)
__global__ void __launch_bounds__(kBudgetThreads)
    budget_boundary_kernel(const BlockDev* __restrict__ tab, double* out,
                           int accumulate) {
  const BlockDev& B = tab[blockIdx.x];
  const int nc[3] = {B.nc1, B.nc2, B.nc3};
  const int ng = B.ng;
  const size_t plane = (size_t)nc[0] * nc[1] * nc[2];
  const double area[3] = {B.dx3 * B.dx2, B.dx3 * B.dx1, B.dx2 * B.dx1};
  int lo[3], nx[3];
  for (int a = 0; a < 3; ++a) {
    lo[a] = nc[a] > 1 ? ng : 0;
    nx[a] = nc[a] > 1 ? nc[a] - 2 * ng : 1;
  }
  double acc[NHYDRO] = {0., 0., 0., 0., 0.};
  for (int d = 0; d < 3; ++d) {
    const double* S = B.step[d];
    if (!S) continue;
    // the two transverse axes of direction d, fastest first
    const int ta = d == 0 ? 1 : 0, tb = d == 2 ? 1 : 2;
    const size_t nt = (size_t)nx[ta] * nx[tb];
    for (int side = 0; side < 2; ++side) {
      const int bc = B.bc[2 * d + side];
      if (bc != kBcReflecting && bc != kBcExtrapolation) continue;
      const double w = (side ? 1. : -1.) * area[d];
      const int f = side ? nc[d] - ng : ng;
      for (size_t e = threadIdx.x; e < nt; e += kBudgetThreads) {
        int idx[3];
        idx[d] = f;
        idx[ta] = lo[ta] + (int)(e % nx[ta]);
        idx[tb] = lo[tb] + (int)(e / nx[ta]);
        const size_t c = ((size_t)idx[2] * nc[1] + idx[1]) * nc[0] + idx[0];
#pragma unroll
        for (int v = 0; v < NHYDRO; ++v) acc[v] += S[v * plane + c] * w;
      }
    }
  }
  budget_reduce(acc, out + NHYDRO * blockIdx.x, accumulate != 0);
}

// the partitioned solve's reciprocal on a device array (a check of its
// error bound against the IEEE division)
__global__ void psw_rcp_kernel(const double* __restrict__ x,
                               double* __restrict__ r, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    r[i] = psw_rcp(x[i]);
}

}  // namespace
}  // namespace sg

using namespace sg;

// ---------------------------------------------------------------------------
// host launchers (called by sg_api.cpp); all asynchronous on `stream`
// ---------------------------------------------------------------------------
extern "C" size_t SG_NAME(sg_stage_smem)(int nc1, int tj, int has2, int wb,
                                          int cov, int visc) {
  TileLayout L(tj, nc1, 3, has2 != 0, wb != 0, cov != 0, visc != 0);
  return (size_t)L.total * sizeof(real);
}

extern "C" int SG_NAME(sg_launch_stage)(const BlockDev* tab, StageParams p,
                                        size_t smem, cudaStream_t stream) {
#ifdef SG_REAL_IS_FLOAT
  // the FP32 reference's base parts, from the base as it is now
  if (p.ref32) base_ref_kernel<<<p.nblock, 32, 0, stream>>>(tab);
#endif
  void (*k)(const BlockDev*, StageParams) = nullptr;
  if (p.riemann == kHllc)
    k = p.shock ? stage_kernel<kHllc, true> : stage_kernel<kHllc, false>;
  else
    k = p.shock ? stage_kernel<kLmars, true> : stage_kernel<kLmars, false>;
  // the opt-in shared memory is raised once per kernel, to the largest size
  // any handle asked for (never inside a stream capture: the first launch of
  // a handle is eager)
  static size_t granted[4] = {0, 0, 0, 0};
  size_t& g = granted[(p.riemann == kHllc ? 0 : 2) + (p.shock ? 1 : 0)];
  if (smem > g) {
    cudaError_t e = cudaFuncSetAttribute(
        k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    g = smem;
  }
  // a persistent grid: as many CTAs as fit on the GPU at once, never more
  // than there are tiles
  static int resident[4][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
  int kid = (p.riemann == kHllc ? 0 : 2) + (p.shock ? 1 : 0);
  if (resident[kid][1] != (int)smem) {
    int per_sm = 0, dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kThreads, smem);
    resident[kid][0] = (per_sm > 0 ? per_sm : 1) * sms;
    resident[kid][1] = (int)smem;
  }
  int grid = p.ntile < resident[kid][0] ? p.ntile : resident[kid][0];
  k<<<grid, kThreads, smem, stream>>>(tab, p);
  return (int)cudaGetLastError();
}

extern "C" int SG_NAME(sg_launch_x3)(const BlockDev* tab, StageParams p,
                                     size_t max_cells, cudaStream_t stream) {
  void (*k)(const BlockDev*, StageParams) = nullptr;
  if (p.riemann == kHllc)
    k = p.shock ? x3_kernel<kHllc, true> : x3_kernel<kHllc, false>;
  else
    k = p.shock ? x3_kernel<kLmars, true> : x3_kernel<kLmars, false>;
  if (p.visc3) {  // viscosity's prep of the 3-D blocks first
    int gv = (int)((max_cells + kThreads - 1) / kThreads);
    if (gv > 2048) gv = 2048;
    visc3_kernel<<<dim3(gv, p.nblock), kThreads, 0, stream>>>(tab, p);
  }
  // threads: cells / kX3Chunk per block (bounded by a few waves)
  size_t work = max_cells / kX3Chunk + 1;
  int gx = (int)((work + kThreads - 1) / kThreads);
  if (gx > 2048) gx = 2048;
  k<<<dim3(gx, p.nblock), kThreads, 0, stream>>>(tab, p);
  return (int)cudaGetLastError();
}

extern "C" int SG_NAME(sg_launch_scalar)(const BlockDev* tab, StageParams p,
                                         size_t max_plane, size_t max_icols,
                                         cudaStream_t stream) {
  int gx = (int)((3 * max_plane + kThreads - 1) / kThreads);
  if (gx > 2048) gx = 2048;
  scalar_flux_kernel<<<dim3(gx, p.nblock), kThreads, 0, stream>>>(tab, p);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return (int)e;
  int gu = (int)((max_plane + kThreads - 1) / kThreads);
  if (gu > 2048) gu = 2048;
  // the positivity limiter (blocks with the covariance row; the others
  // return at once)
  scalar_theta_kernel<<<dim3(gu, p.nblock), kThreads, 0, stream>>>(tab, p);
  scalar_theta_ghost_kernel<<<dim3(gu, p.nblock), kThreads, 0, stream>>>(tab);
  scalar_scale_kernel<<<dim3(gx, p.nblock), kThreads, 0, stream>>>(tab);
  e = cudaGetLastError();
  if (e != cudaSuccess) return (int)e;
  scalar_update_kernel<<<dim3(gu, p.nblock), kThreads, 0, stream>>>(tab, p);
  if (max_icols > 0) {  // implicit blocks: the solve's transfer per column
    e = cudaGetLastError();
    if (e != cudaSuccess) return (int)e;
    const int gv = (int)((16 * max_icols + kVicScalarWarps - 1) / kVicScalarWarps);
    scalar_vic_kernel<<<dim3(gv, p.nblock), 32 * kVicScalarWarps, 0, stream>>>(
        tab, p);
  }
  return (int)cudaGetLastError();
}

extern "C" int SG_NAME(sg_launch_scalar_ghost)(const BlockDev* tab, int nblock,
                                               int which, size_t max_plane,
                                               cudaStream_t stream) {
  int gx = (int)((max_plane + kThreads - 1) / kThreads);
  if (gx > 1024) gx = 1024;
  scalar_ghost_kernel<<<dim3(gx, nblock), kThreads, 0, stream>>>(tab, which);
  return (int)cudaGetLastError();
}

extern "C" int SG_NAME(sg_launch_ghost)(const BlockDev* tab, int nblock,
                                        int which, size_t max_plane,
                                        cudaStream_t stream) {
  int gx = (int)((max_plane + kThreads - 1) / kThreads);
  if (gx > 1024) gx = 1024;
  ghost_kernel<<<dim3(gx, nblock), kThreads, 0, stream>>>(tab, which);
  return (int)cudaGetLastError();
}

extern "C" int SG_NAME(sg_launch_prim)(const BlockDev* tab, int nblock,
                                       int which, void* const* out,
                                       size_t max_plane, cudaStream_t stream) {
  int gx = (int)((max_plane + kThreads - 1) / kThreads);
  if (gx > 1024) gx = 1024;
  prim_kernel<<<dim3(gx, nblock), kThreads, 0, stream>>>(tab, which, out);
  return (int)cudaGetLastError();
}

extern "C" int SG_NAME(sg_launch_init)(const BlockDev* tab, int nblock,
                                       int which, double* const* win,
                                       size_t max_plane, cudaStream_t stream) {
  int gx = (int)((max_plane + kThreads - 1) / kThreads);
  if (gx > 1024) gx = 1024;
  init_kernel<<<dim3(gx, nblock), kThreads, 0, stream>>>(tab, which, win);
  return (int)cudaGetLastError();
}

// the three VIC launches of a stage (after the stage kernel wrote the
// explicit tendency of the implicit blocks)
extern "C" int SG_NAME(sg_launch_vic)(const BlockDev* tab, StageParams p,
                                      size_t max_cells, size_t max_cols,
                                      int wide, int* status,
                                      cudaStream_t stream, cudaEvent_t* ev) {
  int ga = (int)((max_cells + kThreads - 1) / kThreads);
  if (ga > 4096) ga = 4096;
  if (p.asm_kinds & 1)
    vic_assemble_kernel<double><<<dim3(ga, p.nblock), kThreads, 0, stream>>>(tab, p);
#ifdef SG_REAL_IS_FLOAT
  if (p.asm_kinds & 2)
    vic_assemble_kernel<float><<<dim3(ga, p.nblock), kThreads, 0, stream>>>(tab, p);
#endif
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return (int)e;
  if (ev) cudaEventRecord(ev[0], stream);
  // implicit-precision float32 blocks: the FP32 sweep, then the refined
  // solve's corrections (FP64 residuals), or (refine < 0) the FP32 solve's
  // Woodbury step alone; the columns either leaves are solved directly
  int gs = (int)((max_cols + kVicCols - 1) / kVicCols);
  if (p.refine) {
    int gr = (int)((max_cells + kResThreads - 1) / kResThreads);
    if (gr > 4096 * (kThreads / kResThreads)) gr = 4096 * (kThreads / kResThreads);
    const size_t cw = (max_cols + kCorrCols - 1) / kCorrCols;  // warps
    const int gc = (int)((cw + kCorrWarps - 1) / kCorrWarps);
    vic_solve32_kernel<<<dim3(gs, p.nblock), 32, 0, stream>>>(tab, p);
    if (p.refine < 0) {  // the FP32 solve: its Woodbury step, no corrections
      const size_t threads = max_cols * 32;
      const int gw = (int)((threads + kThreads - 1) / kThreads);
      vic_woodbury32_kernel<<<dim3(gw, p.nblock), kThreads, 0, stream>>>(tab, p);
    }
    for (int k = 1; k <= p.refine; ++k) {
      vic_residual_kernel<<<dim3(gr, p.nblock), kResThreads, 0, stream>>>(tab, p, k);
      vic_correct32_kernel<<<dim3(gc, p.nblock), 32 * kCorrWarps, 0, stream>>>(
          tab, p, k == p.refine);
    }
    // the columns left to FP64: the partitioned FP64 solve first (a warp
    // per column, four chunks at once), the serial one for what it cannot
    vic_psolve_kernel<true><<<dim3((unsigned)max_cols, p.nblock), 32, 0, stream>>>(tab, p);
    e = cudaGetLastError();
    if (e != cudaSuccess) return (int)e;
  }
  // the solve: the full matrix kVicCols columns per single-warp CTA, the
  // partial one a thread per column; blocks with the partitioned form take
  // it first (a warp per column), the serial solve then only the columns
  // it marked
  if (p.psw) {
    vic_psolve_kernel<false><<<dim3((unsigned)max_cols, p.nblock), 32, 0, stream>>>(tab, p);
    e = cudaGetLastError();
    if (e != cudaSuccess) return (int)e;
  }
  if (p.vic_kinds & 1) {
    if (p.refine)
      vic_solve_kernel<true><<<dim3(gs, p.nblock), 32, 0, stream>>>(tab, p, status);
    else
      vic_solve_kernel<false><<<dim3(gs, p.nblock), 32, 0, stream>>>(tab, p, status);
  }
  if (p.vic_kinds & 2) {
    const int g3 = (int)((max_cols + kThreads - 1) / kThreads);
    vic_solve3_kernel<<<dim3(g3, p.nblock), kThreads, 0, stream>>>(tab, p, status);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return (int)e;
  if (ev) cudaEventRecord(ev[1], stream);
  if (wide) {
    // three passes: per cell, the serial scans per column, per cell
    int gt = (int)((max_cols + kFinishBThreads - 1) / kFinishBThreads);
    int gc = (int)((max_cells + kThreads - 1) / kThreads);
    if (gc > 8192) gc = 8192;
    vic_finish_a_kernel<<<dim3(gc, p.nblock), kThreads, 0, stream>>>(tab, p);
    vic_finish_b_kernel<<<dim3(gt, p.nblock), kFinishBThreads, 0, stream>>>(tab, p);
    vic_finish_c_kernel<<<dim3(gc, p.nblock), kThreads, 0, stream>>>(tab, p);
  } else {
    int gc = (int)((max_cols + kVicWarps - 1) / kVicWarps);
    vic_finish_kernel<32><<<dim3(gc, p.nblock), 32 * kVicWarps, 0, stream>>>(tab, p);
  }
  return (int)cudaGetLastError();
}

extern "C" int SG_NAME(sg_launch_psw_rcp)(const double* x, double* r,
                                          size_t n, cudaStream_t stream) {
  size_t g = (n + kThreads - 1) / kThreads;
  if (g > 4096) g = 4096;
  psw_rcp_kernel<<<(unsigned)g, kThreads, 0, stream>>>(x, r, n);
  return (int)cudaGetLastError();
}

extern "C" int SG_NAME(sg_launch_reduce)(const BlockDev* tab, int nblock,
                                         int which, unsigned long long* red,
                                         int* flag, size_t max_cells,
                                         cudaStream_t stream) {
  int gx = (int)((max_cells + kThreads - 1) / kThreads);
  if (gx > 64) gx = 64;
  reduce_kernel<<<dim3(gx, nblock), kThreads, 0, stream>>>(tab, which, red,
                                                           flag);
  return (int)cudaGetLastError();
}

extern "C" int SG_NAME(sg_launch_budget_totals)(const BlockDev* tab,
                                                int nblock, int which,
                                                double* out,
                                                cudaStream_t stream) {
  budget_totals_kernel<<<nblock, kBudgetThreads, 0, stream>>>(tab, which, out);
  return (int)cudaGetLastError();
}

extern "C" int SG_NAME(sg_launch_budget_boundary)(const BlockDev* tab,
                                                  int nblock, double* out,
                                                  int accumulate,
                                                  cudaStream_t stream) {
  budget_boundary_kernel<<<nblock, kBudgetThreads, 0, stream>>>(tab, out,
                                                                accumulate);
  return (int)cudaGetLastError();
}
