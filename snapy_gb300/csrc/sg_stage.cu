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

template <int RK>
__device__ __forceinline__ void riemann(const real* wl, const real* wr,
                                        real gammad, int d, real* flx) {
  if (RK == kHllc)
    hllc_flux<real>(wl, wr, gammad, d, flx, nullptr);
  else
    lmars_flux<real>(wl, wr, gammad, d, flx, nullptr);
}

template <int RK, bool SHOCK>
__global__ void __launch_bounds__(kThreads)
    stage_kernel(const BlockDev* __restrict__ tab, StageParams p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  real* sm = reinterpret_cast<real*>(smem_raw);
  const int tile = blockIdx.x;
  const int bi = find_block(tab, p.nblock, tile);
  const BlockDev& B = tab[bi];
  const int t = tile - B.tile0;
  const int nc1 = B.nc1, nc2 = B.nc2, ng = B.ng;
  const int nx1 = nc1 - 2 * ng;
  const bool has2 = nc2 > 1;
  const int hj = has2 ? ng : 0;
  const int j0 = (has2 ? ng : 0) + t * B.tj;
  const int jend = has2 ? nc2 - ng : 1;
  const int ntj = min(B.tj, jend - j0);
  const int R = ntj + 2 * hj;
  const size_t plane = (size_t)nc1 * nc2 * B.nc3;
  const real* __restrict__ uin = static_cast<const real*>(B.buf[p.in]);
  const real* __restrict__ u0 = static_cast<const real*>(B.buf[p.u0]);
  real* uout = static_cast<real*>(B.buf[p.out]);
  const real gammad = real(B.gammad);
  const bool scale = p.scale != 0;

  const int wstride = R * nc1;  // one variable of the W tile
  real* W = sm;
  const int nf1 = nx1 + 1;
  real* F1 = W + NHYDRO * wstride;
  const int f1stride = ntj * nf1;
  real* F2 = F1 + NHYDRO * f1stride;
  const int f2stride = (ntj + 1) * nx1;

  // (1) the tile and its x2 halo, U -> W
  const size_t row0 = (size_t)(j0 - hj) * nc1;
  for (int idx = threadIdx.x; idx < R * nc1; idx += blockDim.x) {
    real uc[NHYDRO], wc[NHYDRO];
#pragma unroll
    for (int v = 0; v < NHYDRO; ++v) uc[v] = uin[v * plane + row0 + idx];
    cons2prim<real>(uc, wc, gammad);
#pragma unroll
    for (int v = 0; v < NHYDRO; ++v) W[v * wstride + idx] = wc[v];
  }
  __syncthreads();

  // (2) x1 faces ng .. nc1-ng of the tile rows
  for (int idx = threadIdx.x; idx < ntj * nf1; idx += blockDim.x) {
    const int jt = idx / nf1, fi = idx - jt * nf1;
    const real* q = W + (hj + jt) * nc1 + ng + fi;
    real wl[NHYDRO], wr[NHYDRO], flx[NHYDRO];
    face_states<SHOCK>(q, wstride, 1, scale, wl, wr);
    riemann<RK>(wl, wr, gammad, 1, flx);
    if ((fi == 0 && B.bc[0] == kBcReflecting) ||
        (fi == nx1 && B.bc[1] == kBcReflecting))
      flx[IDN] = flx[IPR] = real(0);
#pragma unroll
    for (int v = 0; v < NHYDRO; ++v) F1[v * f1stride + idx] = flx[v];
  }

  // (3) x2 faces j0 .. j0+ntj of the tile, x1-interior cells
  if (has2) {
    for (int idx = threadIdx.x; idx < (ntj + 1) * nx1; idx += blockDim.x) {
      const int jf = idx / nx1, ii = idx - jf * nx1;
      const real* q = W + (hj + jf) * nc1 + ng + ii;
      real wl[NHYDRO], wr[NHYDRO], flx[NHYDRO];
      face_states<SHOCK>(q, wstride, nc1, scale, wl, wr);
      riemann<RK>(wl, wr, gammad, 2, flx);
      const int jface = j0 + jf;
      if ((jface == ng && B.bc[2] == kBcReflecting) ||
          (jface == nc2 - ng && B.bc[3] == kBcReflecting))
        flx[IDN] = flx[IPR] = real(0);
#pragma unroll
      for (int v = 0; v < NHYDRO; ++v) F2[v * f2stride + idx] = flx[v];
    }
  }
  __syncthreads();

  // (4) divergence, du = -dt div, RK combine on the interior cells
  const real a1 = real(B.dx3 * B.dx2), a2 = real(B.dx3 * B.dx1);
  const real vol = real(B.dx3 * (B.dx2 * B.dx1));
  const real mdt = real(-p.dt[bi]);
  const real w0 = real(p.w0), w1 = real(p.w1), w2 = real(p.w2);
  for (int idx = threadIdx.x; idx < ntj * nx1; idx += blockDim.x) {
    const int jt = idx / nx1, ii = idx - jt * nx1;
    const size_t c = (size_t)(j0 + jt) * nc1 + ng + ii;
#pragma unroll
    for (int v = 0; v < NHYDRO; ++v) {
      const real* f1 = F1 + v * f1stride + jt * nf1 + ii;
      real dv = a1 * f1[1] - a1 * f1[0];
      if (has2) {
        const real* f2 = F2 + v * f2stride + jt * nx1 + ii;
        dv = dv + (a2 * f2[nx1] - a2 * f2[0]);
      }
      real du = mdt * (dv / vol);
      const size_t q = v * plane + c;
      uout[q] = w0 * u0[q] + w1 * uin[q] + w2 * du;
    }
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
    cons2prim<real>(uc, wc, gammad);
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
    cons2prim<real>(uc, w, gammad);
    const real cs = sqrt(gammad * w[IPR] / w[IDN]);
    if (nc1 > 1) dtm = fmin(dtm, (double)(real(B.dx1) / (fabs(w[IVX]) + cs)));
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
    atomicMin(&red[4 * b + 0], key(dtm));
    atomicMin(&red[4 * b + 1], key(rmin));
    atomicMin(&red[4 * b + 2], key(pmin));
    if (nan) atomicOr(&flag[b], 1);
  }
}

}  // namespace
}  // namespace sg

using namespace sg;

// ---------------------------------------------------------------------------
// host launchers (called by sg_api.cpp); all asynchronous on `stream`
// ---------------------------------------------------------------------------
extern "C" size_t SG_NAME(sg_stage_smem)(int nc1, int nx1, int tj, int has2) {
  int hj = has2 ? 3 : 0;
  size_t w = (size_t)NHYDRO * (tj + 2 * hj) * nc1;
  size_t f1 = (size_t)NHYDRO * tj * (nx1 + 1);
  size_t f2 = has2 ? (size_t)NHYDRO * (tj + 1) * nx1 : 0;
  return (w + f1 + f2) * sizeof(real);
}

extern "C" int SG_NAME(sg_launch_stage)(const BlockDev* tab, StageParams p,
                                        size_t smem, cudaStream_t stream) {
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
  k<<<p.ntile, kThreads, smem, stream>>>(tab, p);
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
