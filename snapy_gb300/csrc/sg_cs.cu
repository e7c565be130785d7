// The cubed-sphere shallow-water stage: six gnomonic-equiangle panels of
// n x n cells (nghost 3, one radial cell) in ONE handle, FP64 or FP32 state
// (6, 4, nc, nc): Phi, the radial and the two covariant tangential momenta.
//
// A stage is five launches, each over all six panels:
//   cs_flux_kernel       every x2 and x3 face of the panels' interiors: the
//                        primitives of its six-cell stencil (U/Phi, momenta
//                        raised by the cell cosine), weno5 for Phi and cp5
//                        for the velocities, the face-frame rotation, the
//                        shallow-roe flux (dir yz) and its rotation back to
//                        covariant components
//                        (src/riemann/riemann.cpp:219-346 with
//                        src/coord/gnomonic_equiangle.cpp:357-463,
//                        src/riemann/riemann_kernels.h:447-495)
//                        (a seam face keeps its interior-side state)
//   cs_seam_face_kernel  the seam faces again, each with its exterior-side
//                        state the neighbour panel's own interior-side
//                        state, mapped into this panel's frame at the
//                        shared face (the cross-panel face-state sync,
//                        src/hydro/hydro_forward.cpp:719-757)
//   cs_seam_flux_kernel  the seam faces of the non-owning panels take the
//                        owner's flux through the Cartesian frame
//                        (src/layout/seam_register.cpp:35)
//   cs_update_kernel     (A2 dF2 + A3 dF3) / V minus the metric sources,
//                        du = -dt div, and the RK combine
//                        (src/coord/coordinate.cpp:618-662,
//                        src/coord/gnomonic_equiangle.cpp:465-521)
//   cs_ghost_kernel      the seam halo: a gather along the neighbour's edge
//                        row with the momenta through each point's local
//                        geographic frame (r, theta, phi)
//                        (src/layout/cubed_sphere_layout.cpp:563-803,
//                        src/coord/gnomonic_equiangle.cpp:536-609)
// All the seam geometry is in three tables built once on the host; the
// kernels only gather.  This file is compiled twice: as the host API with
// the FP64 kernels, built with -fmad=false (the oracle's operations in its
// order), and with SG_CS_F32_UNIT defined as the FP32 kernels alone, with
// contraction allowed (the FP32 path is held to a tolerance, not to the
// oracle's rounding); the host calls those through cs_f32_*.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>

#include <string>

#include "../../include/snapy_gb300.h"
#include "sg_device.cuh"

extern "C" int sg_fail_message(int code, const char* msg);

// the launch parameters of every kernel, shared by the two translation units
namespace sgcs {
struct CsParams {
  int n, nc;
  // the geometry, the ghost table and the seam table in the state's type
  const void* geo;
  const void* gtab;
  int nghost;
  const void* stab;
  int nseam;
  const void* sst;  // the seam face-state table (4 sides x n per panel)
  void* sbuf;       // the seam faces' interior-side states (24 n x 4)
  const void* in;
  const void* u0;
  void* out;
  void* f2;
  void* f3;
  const double* dt;
  double w0, w1, w2;
  double phi0;  // FP32: the reference geopotential of the pressure anomaly
  int hllc;     // 1: HLLC for shallow water, 0: shallow-roe (dir yz)
  // the FluxRegister's step fields S_2, S_3 (FP64, laid out as f2 / f3;
  // null: not requested), the FP64 geometry, and whether this is stage 0
  double* s2;
  double* s3;
  const void* geo64;
  int first;
};

// the FP32 launches, defined in the FP32 unit
int f32_stage(const CsParams& P, size_t faces, size_t cells, cudaStream_t s);
int f32_ghost(const CsParams& P, void* buf, cudaStream_t s);
int f32_dt(const CsParams& P, const void* buf, unsigned long long* key, int g,
           cudaStream_t s);
}  // namespace sgcs

namespace {

using sg::IDN;
using sg::IVX;
using sg::IVY;
using sg::IVZ;
using sg::as_f64;

constexpr int kThreads = 256;
constexpr int kNg = 3;
constexpr int kGhostStride = 24;
constexpr int kSeamStride = 18;
constexpr int kSeamStateStride = 16;

// offsets of the geometry arrays in the device block (see sg_cs_desc); the
// FP32 kernels read an FP32 copy made at sg_cs_create (the same values their
// per-use conversions gave, without a conversion per use)
template <typename T>
struct Geo {
  const T *cos_c, *sin_c, *vol, *xr, *yr, *w2, *w3;
  const T *cos_f2, *sin_f2, *a2, *cos_f3, *sin_f3, *a3;
};

template <typename T>
__host__ __device__ inline Geo<T> geo_of(const void* gv, int nc) {
  const T* g = static_cast<const T*>(gv);
  const size_t c = (size_t)nc * nc, f = (size_t)nc * (nc + 1);
  Geo<T> o;
  o.cos_c = g;
  o.sin_c = g + c;
  o.vol = g + 2 * c;
  o.xr = g + 3 * c;
  o.yr = g + 4 * c;
  o.w2 = g + 5 * c;
  o.w3 = g + 6 * c;
  o.cos_f2 = g + 7 * c;
  o.sin_f2 = o.cos_f2 + f;
  o.a2 = o.sin_f2 + f;
  o.cos_f3 = o.a2 + f;
  o.sin_f3 = o.cos_f3 + f;
  o.a3 = o.sin_f3 + f;
  return o;
}

using sgcs::CsParams;

// U -> W of one cell: v = m / Phi, the tangential pair raised by cos.
// With phi0 > 0 (the FP32 state) the stored Phi row is the anomaly
// Phi - phi0: w[IDN] stays the anomaly (what the reconstruction reads) and
// the velocities divide by the total
template <typename T>
__device__ __forceinline__ void sw_prim(const T* q, size_t pst, size_t c,
                                        T cs, T* w, T phi0 = T(0)) {
  const T phi = phi0 > T(0) ? phi0 + q[c] : q[c];
  w[IDN] = q[c];
  const T v1 = q[pst + c] / phi, v2 = q[2 * pst + c] / phi,
          v3 = q[3 * pst + c] / phi;
  const T sth2 = T(1.) - cs * cs;
  w[IVX] = v1;
  w[IVY] = v2 / sth2 - v3 * cs / sth2;
  w[IVZ] = -v2 * cs / sth2 + v3 / sth2;
}

// shallow_roe_impl with dir yz: DIM 2 (x2 faces, normal IVY) or 1 (x3).
// phi0 > 0 (the FP32 state): L[0], R[0] are the anomalies Phi' = Phi - phi0
// the state stores, the totals are formed for the wave speeds and the mass
// flux, and the normal momentum flux carries the pressure anomaly
// phi0 Phi' + Phi'^2 / 2 in place of Phi^2 / 2: the constant phi0^2 / 2 it
// leaves out has no divergence once the metric source leaves it out too
// (the lake at rest), and FP32 would lose the anomaly under it
template <typename T, int DIM>
__device__ __forceinline__ void shallow_roe(const T* L, const T* R, T* F,
                                            T phi0) {
  constexpr int ivx = DIM == 2 ? IVY : IVZ, ivy = DIM == 2 ? IVZ : IVY,
                ivz = IVX;
  // Phi of the two sides (the anomalies L[0], R[0] plus phi0 when phi0 > 0)
  const T pL = phi0 > T(0) ? phi0 + L[0] : L[0];
  const T pR = phi0 > T(0) ? phi0 + R[0] : R[0];
  T sqrtdl = sqrt(pL), sqrtdr = sqrt(pR);
  T isdlpdr = T(1.) / (sqrtdl + sqrtdr);
  T ubar = (L[ivx] * sqrtdl + R[ivx] * sqrtdr) * isdlpdr;
  T vbar = (L[ivy] * sqrtdl + R[ivy] * sqrtdr) * isdlpdr;
  T cbar = sqrt(T(0.5) * (pL + pR));
  T del0 = R[0] - L[0], delx = R[ivx] - L[ivx], dely = R[ivy] - L[ivy];
  T hbar = sqrt(pL * pR);
  T a1 = T(0.5) * (cbar * del0 - hbar * delx) / cbar;
  T a2 = hbar * dely;
  T a3 = T(0.5) * (cbar * del0 + hbar * delx) / cbar;
  T w0[4] = {0, 0, 0, 0}, w1[4] = {0, 0, 0, 0}, w2[4] = {0, 0, 0, 0};
  w0[0] = a1;
  w0[ivx] = a1 * (ubar - cbar);
  w0[ivy] = a1 * vbar;
  w1[ivy] = a2;
  w2[0] = a3;
  w2[ivx] = a3 * (ubar + cbar);
  w2[ivy] = a3 * vbar;
  T s0 = fabs(ubar - cbar), s1 = fabs(ubar), s2 = fabs(ubar + cbar);
  if (phi0 > T(0)) {
    const T dl = L[0], dr = R[0];
    const T ql = phi0 * dl + T(0.5) * dl * dl, qr = phi0 * dr + T(0.5) * dr * dr;
    F[0] = T(0.5) * (pL * L[ivx] + pR * R[ivx]);
    F[ivx] = T(0.5) * (pL * L[ivx] * L[ivx] + ql + pR * R[ivx] * R[ivx] + qr);
    F[ivy] = T(0.5) * (pL * L[ivx] * L[ivy] + pR * R[ivx] * R[ivy]);
  } else {
    F[0] = T(0.5) * (L[0] * L[ivx] + R[0] * R[ivx]);
    F[ivx] = T(0.5) * (L[0] * L[ivx] * L[ivx] + T(0.5) * L[0] * L[0] +
                       R[0] * R[ivx] * R[ivx] + T(0.5) * R[0] * R[0]);
    F[ivy] = T(0.5) * (L[0] * L[ivx] * L[ivy] + R[0] * R[ivx] * R[ivy]);
  }
  F[ivz] = 0;
#pragma unroll
  for (int v = 0; v < 4; ++v)
    F[v] -= T(0.5) * (s0 * w0[v] + s1 * w1[v] + s2 * w2[v]);
}

// HLLC for shallow water in geopotential form (Toro 2001, ch. 10): Davis /
// Einfeldt wave speeds S_L = min(u_L - c_L, u_R - c_R), S_R = max(u_L + c_L,
// u_R + c_R) with c = sqrt(Phi), HLL for Phi and the normal momentum, the
// tangential momentum upwinded across the contact S*.  The reference has no
// shallow-water HLLC; the oracle's og_hllc_sw_batch is its checker.  phi0 as
// in shallow_roe (a constant in the normal momentum flux passes through HLL
// unchanged, so its anomaly form is exact).
template <typename T, int DIM>
__device__ __forceinline__ void hllc_sw(const T* L, const T* R, T* F, T phi0) {
  constexpr int ivx = DIM == 2 ? IVY : IVZ, ivy = DIM == 2 ? IVZ : IVY,
                ivz = IVX;
  const T hL = phi0 > T(0) ? phi0 + L[0] : L[0];
  const T hR = phi0 > T(0) ? phi0 + R[0] : R[0];
  const T cl = sqrt(hL), cr = sqrt(hR);
  const T ul = L[ivx], ur = R[ivx];
  const T sl = fmin(ul - cl, ur - cr), sr = fmax(ul + cl, ur + cr);
  const T ml = hL * ul, mr = hR * ur;
  const T fl0 = ml, fr0 = mr;
  T pl, pr;
  if (phi0 > T(0)) {
    const T dl = L[0], dr = R[0];
    pl = phi0 * dl + T(0.5) * dl * dl;
    pr = phi0 * dr + T(0.5) * dr * dr;
  } else {
    pl = T(0.5) * L[0] * L[0];
    pr = T(0.5) * R[0] * R[0];
  }
  const T fl1 = ml * ul + pl, fr1 = mr * ur + pr;
  T f0, f1, f2;
  if (sl >= T(0)) {
    f0 = fl0;
    f1 = fl1;
    f2 = fl0 * L[ivy];
  } else if (sr <= T(0)) {
    f0 = fr0;
    f1 = fr1;
    f2 = fr0 * R[ivy];
  } else {
    const T inv = T(1.) / (sr - sl);
    f0 = (sr * fl0 - sl * fr0 + sl * sr * (R[0] - L[0])) * inv;
    f1 = (sr * fl1 - sl * fr1 + sl * sr * (mr - ml)) * inv;
    const T den = hR * (ur - sr) - hL * (ul - sl);
    const T ss = (sl * hR * (ur - sr) - sr * hL * (ul - sl)) / den;
    f2 = ss >= T(0) ? f0 * L[ivy] : f0 * R[ivy];
  }
  F[0] = f0;
  F[ivx] = f1;
  F[ivy] = f2;
  F[ivz] = T(0);
}

// the flux of one face: panel p, an x2 face (row k, face j) or an x3 face
// (face k, column j).  The bulk pass (SEAM false) reconstructs both sides
// from the panel's own stencil; at a seam face (side >= 0: side L R B T of
// the panel, `along` its index on that side) it also keeps its interior-side
// state in the seam buffer.  The seam pass (SEAM true) takes the face's own
// interior-side state and the neighbour's from that buffer, the neighbour's
// velocities mapped into this panel's frame at the shared face (the
// reference's cross-panel face-state sync), and redoes the flux
template <typename T, bool HLLC, bool SEAM>
__device__ __forceinline__ void cs_face(const CsParams& P, const Geo<T>& G,
                                        int p, bool x2, int k, int j,
                                        int side, int along) {
  const int n = P.n, nc = P.nc;
  const size_t pst = (size_t)nc * nc;  // one variable of a panel
  const T phi0 = T(P.phi0);
  const T* U = static_cast<const T*>(P.in);
  T* SB = static_cast<T*>(P.sbuf);  // 4 values per seam face
  {
    T wl[4], wr[4], F[4];
    if (!SEAM) {
      const T* q = U + (size_t)p * 4 * pst;
      T st[6][4];
#pragma unroll
      for (int m = 0; m < 6; ++m) {
        const int kk = x2 ? k : k - 3 + m, jj = x2 ? j - 3 + m : j;
        const size_t c = (size_t)kk * nc + jj;
        sw_prim<T>(q, pst, c, T(G.cos_c[c]), st[m], phi0);
      }
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        if (v == IDN) {
          wl[v] = sg::weno5_cp<T>(st[0][v], st[1][v], st[2][v], st[3][v], st[4][v], false);
          wr[v] = sg::weno5_cm<T>(st[1][v], st[2][v], st[3][v], st[4][v], st[5][v], false);
        } else {
          wl[v] = sg::cp5_cp<T>(st[0][v], st[1][v], st[2][v], st[3][v], st[4][v]);
          wr[v] = sg::cp5_cm<T>(st[1][v], st[2][v], st[3][v], st[4][v], st[5][v]);
        }
      }
      if (side >= 0) {  // the interior side: the right one on L / B
        const T* in = (side == 0 || side == 2) ? wr : wl;
        T* b = SB + ((size_t)(p * 4 + side) * n + along) * 4;
#pragma unroll
        for (int v = 0; v < 4; ++v) b[v] = in[v];
      }
    } else {
      const size_t own = (size_t)(p * 4 + side) * n + along;
      const T* r = static_cast<const T*>(P.sst) + own * kSeamStateStride;
      const size_t nb = ((size_t)((int)r[0] * 4 + (int)r[1])) * n + (int)r[2];
      const T* M = r + 4;
      T* in = (side == 0 || side == 2) ? wr : wl;
      T* ext = (side == 0 || side == 2) ? wl : wr;
      T we[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        in[v] = SB[own * 4 + v];
        we[v] = SB[nb * 4 + v];
      }
      ext[IDN] = we[IDN];
#pragma unroll
      for (int a = 0; a < 3; ++a)
        ext[IVX + a] = (M[3 * a] * we[IVX] + M[3 * a + 1] * we[IVY]) +
                       M[3 * a + 2] * we[IVZ];
    }
    const size_t fidx = x2 ? (size_t)k * (nc + 1) + j : (size_t)k * nc + j;
    const T cs = T(x2 ? G.cos_f2[fidx] : G.cos_f3[fidx]);
    const T sn = T(x2 ? G.sin_f2[fidx] : G.sin_f3[fidx]);
    const T gi = T(1.0) / (sn * sn);
    // to the face-local orthonormal frame (prim2local2_ / 3_)
    auto to_face = [&](T* w) {
      const T uu2 = w[IVY], uu3 = w[IVZ];
      if (x2) {
        const T T22 = T(1.0) / sqrt(gi), T32 = cs / sqrt(T(1.0)),
                T33 = sqrt(T(1.0));
        w[IVZ] = T32 * uu2 + T33 * uu3;
        w[IVY] = T22 * uu2;
      } else {
        const T T22 = sqrt(T(1.0)), T23 = cs / sqrt(T(1.0)),
                T33 = T(1.0) / sqrt(gi);
        w[IVY] = T22 * uu2 + T23 * uu3;
        w[IVZ] = T33 * uu3;
      }
    };
    to_face(wl);
    to_face(wr);
    if (HLLC) {
      if (x2)
        hllc_sw<T, 2>(wl, wr, F, phi0);
      else
        hllc_sw<T, 1>(wl, wr, F, phi0);
    } else {
      if (x2)
        shallow_roe<T, 2>(wl, wr, F, phi0);
      else
        shallow_roe<T, 1>(wl, wr, F, phi0);
    }
    // back to covariant fluxes (flux2global2_ / 3_)
    const T txy = F[IVY], txz = F[IVZ];
    if (x2) {
      const T T22 = sqrt(gi), T32 = -sqrt(gi) * cs / T(1.0),
              T33 = T(1.0) / sqrt(T(1.0));
      F[IVZ] = T32 * txy + T33 * txz;
      F[IVY] = T22 * txy;
    } else {
      const T T22 = T(1.0) / sqrt(T(1.0)), T23 = -cs / T(1.0) * sqrt(gi),
              T33 = sqrt(gi);
      F[IVY] = T22 * txy + T23 * txz;
      F[IVZ] = T33 * txz;
    }
    const T ty = F[IVY], tz = F[IVZ];
    F[IVY] = ty + tz * cs;
    F[IVZ] = tz + ty * cs;
    T* out = static_cast<T*>(x2 ? P.f2 : P.f3);
    const size_t fst = (size_t)nc * (nc + 1);  // one variable of a panel's faces
#pragma unroll
    for (int v = 0; v < 4; ++v) out[((size_t)p * 4 + v) * fst + fidx] = F[v];
  }
}

// the faces: thread e < 6 n (n + 1) an x2 face (panel, row k, face j), the
// rest x3 faces (panel, face k, column j), each from its own panel's
// stencils; a seam face keeps its interior-side state for the seam pass
template <typename T, bool HLLC>
__global__ void __launch_bounds__(kThreads)
    cs_flux_kernel(const __grid_constant__ CsParams P) {
  const int n = P.n;
  const Geo<T> G = geo_of<T>(P.geo, P.nc);
  const size_t nf = (size_t)6 * n * (n + 1);
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < 2 * nf;
       e += (size_t)gridDim.x * blockDim.x) {
    const bool x2 = e < nf;
    const size_t r = x2 ? e : e - nf;
    int p, k, j, side = -1, along = 0;
    if (x2) {  // faces j = ng..ng+n of rows k = ng..ng+n-1
      j = kNg + (int)(r % (n + 1));
      k = kNg + (int)((r / (n + 1)) % n);
      p = (int)(r / ((size_t)(n + 1) * n));
      if (j == kNg || j == kNg + n) side = j == kNg ? 0 : 1, along = k - kNg;
    } else {  // faces k = ng..ng+n of columns j = ng..ng+n-1
      j = kNg + (int)(r % n);
      k = kNg + (int)((r / n) % (n + 1));
      p = (int)(r / ((size_t)n * (n + 1)));
      if (k == kNg || k == kNg + n) side = k == kNg ? 2 : 3, along = j - kNg;
    }
    cs_face<T, HLLC, false>(P, G, p, x2, k, j, side, along);
  }
}

// the 24 n seam faces again from the seam buffer (thread e: panel e / 4n,
// side (e / n) % 4 in L R B T, along e % n): the Riemann problem of the
// face's own interior side and the neighbour's
template <typename T, bool HLLC>
__global__ void __launch_bounds__(kThreads)
    cs_seam_face_kernel(const __grid_constant__ CsParams P) {
  const int n = P.n;
  const Geo<T> G = geo_of<T>(P.geo, P.nc);
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < 24 * n;
       e += gridDim.x * blockDim.x) {
    const int along = e % n, side = (e / n) % 4, p = e / (4 * n);
    const bool x2 = side < 2;
    const int edge = (side & 1) ? kNg + n : kNg;
    const int k = x2 ? kNg + along : edge, j = x2 ? edge : kNg + along;
    cs_face<T, HLLC, true>(P, G, p, x2, k, j, side, along);
  }
}

// the owner's covariant flux pair raised at its face and projected on the
// destination face's tangents, signed
template <typename T>
__global__ void __launch_bounds__(kThreads) cs_seam_flux_kernel(CsParams P) {
  const int nc = P.nc;
  const size_t fst = (size_t)nc * (nc + 1);
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < P.nseam;
       e += gridDim.x * blockDim.x) {
    const T* r = static_cast<const T*>(P.stab) + (size_t)e * kSeamStride;
    T* dst = static_cast<T*>((int)r[0] == 2 ? P.f2 : P.f3);
    const T* src = static_cast<const T*>((int)r[2] == 2 ? P.f2 : P.f3);
    const size_t di = (size_t)r[1], si = (size_t)r[3];
    const size_t dp = di / fst, dc = di % fst, sp = si / fst, sc = si % fst;
    auto at = [&](const T* a, size_t pn, int v, size_t c) {
      return a[(pn * 4 + v) * fst + c];
    };
    const T sign = T(r[4]), c = T(r[5]);
    const T m2 = at(src, sp, IVY, sc), m3 = at(src, sp, IVZ, sc);
    const T s2 = T(1.) - c * c;
    const T v2 = m2 / s2 - m3 * c / s2;
    const T v3 = -m2 * c / s2 + m3 / s2;
    T V[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) V[q] = T(r[6 + q]) * v2 + T(r[9 + q]) * v3;
    const T fd = at(src, sp, IDN, sc), fr = at(src, sp, IVX, sc);
    const T y = (V[0] * T(r[12]) + V[1] * T(r[13])) + V[2] * T(r[14]);
    const T z = (V[0] * T(r[15]) + V[1] * T(r[16])) + V[2] * T(r[17]);
    dst[(dp * 4 + IDN) * fst + dc] = sign * fd;
    dst[(dp * 4 + IVX) * fst + dc] = sign * fr;
    dst[(dp * 4 + IVY) * fst + dc] = sign * y;
    dst[(dp * 4 + IVZ) * fst + dc] = sign * z;
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads) cs_update_kernel(CsParams P) {
  const int n = P.n, nc = P.nc;
  const size_t pst = (size_t)nc * nc, f2st = (size_t)nc * (nc + 1),
               f3st = (size_t)(nc + 1) * nc;
  const Geo<T> G = geo_of<T>(P.geo, nc);
  const T phi0 = T(P.phi0);
  const T* U = static_cast<const T*>(P.in);
  const T* U0 = static_cast<const T*>(P.u0);
  T* O = static_cast<T*>(P.out);
  const T* F2 = static_cast<const T*>(P.f2);
  const T* F3 = static_cast<const T*>(P.f3);
  const T mdt = T(-P.dt[0]);
  const T w0 = T(P.w0), w1 = T(P.w1), w2 = T(P.w2);
  const size_t total = (size_t)6 * n * n;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const int j = kNg + (int)(e % n);
    const int k = kNg + (int)((e / n) % n);
    const int p = (int)(e / ((size_t)n * n));
    const size_t c = (size_t)k * nc + j;
    const T* q = U + (size_t)p * 4 * pst;
    T w[4];
    sw_prim<T>(q, pst, c, T(G.cos_c[c]), w, phi0);
    const size_t i2 = (size_t)k * (nc + 1) + j, i3 = (size_t)k * nc + j;
    const T a2lo = T(G.a2[i2]), a2hi = T(G.a2[i2 + 1]);
    const T a3lo = T(G.a3[i3]), a3hi = T(G.a3[i3 + nc]);
    const T vol = T(G.vol[c]);
    T div[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const T* f2 = F2 + ((size_t)p * 4 + v) * f2st;
      const T* f3 = F3 + ((size_t)p * 4 + v) * f3st;
      const T d2 = a2hi * f2[i2 + 1] - a2lo * f2[i2];
      const T d3 = a3hi * f3[i3 + nc] - a3lo * f3[i3];
      div[v] = (d2 + d3) / vol;
    }
    // Phi and p = Phi^2 / 2; with phi0 > 0, the stored anomaly Phi' and
    // the pressure anomaly phi0 Phi' + Phi'^2 / 2 (see shallow_roe)
    T rho = w[IDN], pr = T(0.5) * (w[IDN] * w[IDN]);
    if (phi0 > T(0)) {
      const T dp = w[IDN];
      rho = phi0 + dp;
      pr = phi0 * dp + T(0.5) * dp * dp;
    }
    const T sn = T(G.sin_c[c]);
    const T sine2 = sn * sn;
    div[IVY] -= T(G.xr[c]) * (pr + rho * w[IVZ] * w[IVZ] * sine2);
    div[IVZ] -= T(G.yr[c]) * (pr + rho * w[IVY] * w[IVY] * sine2);
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const size_t qi = ((size_t)p * 4 + v) * pst + c;
      const T du = mdt * div[v];
      O[qi] = w0 * U0[qi] + w1 * U[qi] + w2 * du;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads) cs_ghost_kernel(CsParams P, void* buf) {
  const int nc = P.nc;
  const size_t pst = (size_t)nc * nc;
  T* Q = static_cast<T*>(buf);
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < P.nghost;
       e += gridDim.x * blockDim.x) {
    const T* r = static_cast<const T*>(P.gtab) + (size_t)e * kGhostStride;
    const size_t d = (size_t)r[0], s0 = (size_t)r[1], s1 = (size_t)r[2];
    // flat (panel, k, j) -> the variable v of that cell
    auto at = [&](size_t f, int v) -> size_t {
      return ((f / pst) * 4 + v) * pst + f % pst;
    };
    const T x = T(r[3]);
#pragma unroll
    for (int v = IDN; v <= IVX; ++v) {
      const T a = Q[at(s0, v)], b = Q[at(s1, v)];
      Q[at(d, v)] = a + x * (b - a);
    }
    T V0[3], V1[3];
    const size_t src[2] = {s0, s1};
    T* Vs[2] = {V0, V1};
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const T* g = r + 4 + 7 * s;
      const T c = T(g[0]);
      const T m2 = Q[at(src[s], IVY)], m3 = Q[at(src[s], IVZ)];
      const T s2 = T(1.) - c * c;
      const T v2 = m2 / s2 - m3 * c / s2;
      const T v3 = -m2 * c / s2 + m3 / s2;
#pragma unroll
      for (int qq = 0; qq < 3; ++qq) Vs[s][qq] = T(g[1 + qq]) * v2 + T(g[4 + qq]) * v3;
    }
    T V[3];
#pragma unroll
    for (int qq = 0; qq < 3; ++qq) V[qq] = V0[qq] + x * (V1[qq] - V0[qq]);
    Q[at(d, IVY)] = (V[0] * T(r[18]) + V[1] * T(r[19])) + V[2] * T(r[20]);
    Q[at(d, IVZ)] = (V[0] * T(r[21]) + V[1] * T(r[22])) + V[2] * T(r[23]);
  }
}

// order-preserving keys of doubles for an unsigned atomicMin
constexpr unsigned long long kKeyInf = 0xfff0000000000000ull;  // key(+inf)
__device__ __forceinline__ unsigned long long dkey(double x) {
  unsigned long long k = __double_as_longlong(x);
  return (k >> 63) ? ~k : (k | 0x8000000000000000ull);
}
__device__ __forceinline__ double dunkey(unsigned long long k) {
  return __longlong_as_double((k >> 63) ? (k & 0x7fffffffffffffffull) : ~k);
}

// min over the interior of width / (|v| + sqrt(Phi)) on x2 and x3
template <typename T>
__global__ void __launch_bounds__(kThreads) cs_dt_kernel(CsParams P, const void* buf,
                                                         unsigned long long* key) {
  const int n = P.n, nc = P.nc;
  const size_t pst = (size_t)nc * nc;
  const Geo<T> G = geo_of<T>(P.geo, nc);
  const T phi0 = T(P.phi0);
  const T* U = static_cast<const T*>(buf);
  // the minimum in the state's type, widened once per warp (exact and
  // monotone, so the same value as widening every cell)
  T m = T(INFINITY);
  int nan = 0;
  const size_t total = (size_t)6 * n * n;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const int j = kNg + (int)(e % n);
    const int k = kNg + (int)((e / n) % n);
    const int p = (int)(e / ((size_t)n * n));
    const size_t c = (size_t)k * nc + j;
    T w[4];
    sw_prim<T>(U + (size_t)p * 4 * pst, pst, c, T(G.cos_c[c]), w, phi0);
    const T cs = sqrt(phi0 > T(0) ? phi0 + w[IDN] : w[IDN]);
    const T d2 = T(G.w2[c]) / (fabs(w[IVY]) + cs);
    const T d3 = T(G.w3[c]) / (fabs(w[IVZ]) + cs);
    if (isnan(d2) || isnan(d3)) nan = 1;
    m = fmin(m, fmin(d2, d3));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    m = fmin(m, __shfl_xor_sync(0xffffffffu, m, o));
    nan |= __shfl_xor_sync(0xffffffffu, nan, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&key[0], dkey((double)m));
    if (nan) atomicOr(&key[1], 1ull);
  }
}

// dt = cfl min (NaN if any cell was), and the keys reset for the next call
__global__ void cs_dt_finish(unsigned long long* key, double cfl, double* dt) {
  dt[0] = key[1] ? __longlong_as_double(0x7ff8000000000000ll)
                 : cfl * dunkey(key[0]);
  key[0] = kKeyInf;
  key[1] = 0;
}

// the budget's row totals (BudgetConsumer, src/diagnostics/budget.cpp:68-200):
// sum over the interior cells of u V per variable, in FP64, an FP32 state's
// Phi row with its reference added back; one CTA, a fixed stride and a
// fixed tree, so the sums are the same on every run
constexpr int kBudgetThreads = 256;
template <typename T>
__global__ void __launch_bounds__(kBudgetThreads)
    cs_budget_kernel(CsParams P, const void* buf, double* out) {
  __shared__ double red[4][kBudgetThreads];
  const int n = P.n, nc = P.nc;
  const size_t pst = (size_t)nc * nc;
  const Geo<double> G = geo_of<double>(P.geo64, nc);
  const T* U = static_cast<const T*>(buf);
  double acc[4] = {0., 0., 0., 0.};
  const size_t total = (size_t)6 * n * n;
  for (size_t e = threadIdx.x; e < total; e += kBudgetThreads) {
    const int j = kNg + (int)(e % n), k = kNg + (int)((e / n) % n);
    const int p = (int)(e / ((size_t)n * n));
    const size_t c = (size_t)k * nc + j;
    const double vol = G.vol[c];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      double u = as_f64(U[((size_t)p * 4 + v) * pst + c]);
      if (v == IDN && P.phi0 > 0.) u = P.phi0 + u;
      acc[v] += u * vol;
    }
  }
#pragma unroll
  for (int v = 0; v < 4; ++v) red[v][threadIdx.x] = acc[v];
  __syncthreads();
  for (int h = kBudgetThreads / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h)
#pragma unroll
      for (int v = 0; v < 4; ++v) red[v][threadIdx.x] += red[v][threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x < 4) out[threadIdx.x] = red[threadIdx.x][0];
}

thread_local std::string g_cs_err;

int cs_fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return sg_fail_message(code, buf);
}

int grid_for(size_t work) {
  size_t g = (work + kThreads - 1) / kThreads;
  if (g > 4096) g = 4096;
  return (int)(g ? g : 1);
}

// the step fields (FluxRegister::end_stage, src/hydro/flux_register.hpp
// :241-402): S_d <- w1 S_d + w2 dt T_d on every interior face of both
// directions, in FP64, from the stage's final face fluxes (the seam faces
// single-valued).  An FP32 state's normal-momentum flux carries the
// pressure anomaly phi0 Phi' + Phi'^2 / 2; the constant phi0^2 / 2 it leaves
// out is added back here in FP64, through the face's rotation to covariant
// components, so S_d means what the FP64 path's does
template <typename T>
__global__ void __launch_bounds__(kThreads) cs_step_kernel(CsParams P) {
  const int n = P.n, nc = P.nc;
  const size_t fst = (size_t)nc * (nc + 1);  // one variable of a panel's faces
  const size_t per = (size_t)n * (n + 1);    // interior faces of one of them
  const double w1 = P.w1, w2dt = P.w2 * P.dt[0];
  const double p0 = 0.5 * (P.phi0 * P.phi0);
  const Geo<double> G = geo_of<double>(P.geo64, nc);
  const size_t total = 2 * (size_t)24 * per;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const bool x2 = e < (size_t)24 * per;
    const size_t r = x2 ? e : e - (size_t)24 * per;
    const int pv = (int)(r / per);  // panel * 4 + variable
    const size_t a = r - (size_t)pv * per;
    const int along = (int)(a % (n + 1)), across = (int)(a / (n + 1));
    const size_t fidx = x2 ? (size_t)(kNg + across) * (nc + 1) + kNg + along
                           : (size_t)(kNg + along) * nc + kNg + across;
    const T* F = static_cast<const T*>(x2 ? P.f2 : P.f3);
    double t = as_f64(F[(size_t)pv * fst + fidx]);
    const int v = pv & 3;
    if (p0 > 0. && v >= IVY) {
      const double cs = x2 ? G.cos_f2[fidx] : G.cos_f3[fidx];
      const double sn = x2 ? G.sin_f2[fidx] : G.sin_f3[fidx];
      const double rg = sqrt(1.0 / (sn * sn));
      // the normal flux's share in (F_IVY, F_IVZ) before the lowering
      const double ty = x2 ? rg * p0 : (-cs * rg) * p0;
      const double tz = x2 ? (-rg * cs) * p0 : rg * p0;
      t += v == IVY ? ty + tz * cs : tz + ty * cs;
    }
    double* S = (x2 ? P.s2 : P.s3) + (size_t)pv * fst + fidx;
    *S = P.first ? fma(w2dt, t, 0.) : fma(w2dt, t, *S * w1);
  }
}

// the five launches of a stage, the seam halo and the dt reduction in T
template <typename T>
int launch_stage(const CsParams& P, size_t faces, size_t cells, cudaStream_t s) {
  (P.hllc ? cs_flux_kernel<T, true> : cs_flux_kernel<T, false>)
      <<<grid_for(faces), kThreads, 0, s>>>(P);
  (P.hllc ? cs_seam_face_kernel<T, true> : cs_seam_face_kernel<T, false>)
      <<<grid_for(24 * (size_t)P.n), kThreads, 0, s>>>(P);
  cs_seam_flux_kernel<T><<<grid_for(P.nseam), kThreads, 0, s>>>(P);
  if (P.s2 && P.s3)
    cs_step_kernel<T><<<grid_for(2 * (size_t)24 * P.n * (P.n + 1)), kThreads, 0, s>>>(P);
  cs_update_kernel<T><<<grid_for(cells), kThreads, 0, s>>>(P);
  cs_ghost_kernel<T><<<grid_for(P.nghost), kThreads, 0, s>>>(P, P.out);
  return (int)cudaGetLastError();
}

template <typename T>
int launch_ghost(const CsParams& P, void* buf, cudaStream_t s) {
  cs_ghost_kernel<T><<<grid_for(P.nghost), kThreads, 0, s>>>(P, buf);
  return (int)cudaGetLastError();
}

template <typename T>
int launch_dt(const CsParams& P, const void* buf, unsigned long long* key,
              int g, cudaStream_t s) {
  cs_dt_kernel<T><<<g, kThreads, 0, s>>>(P, buf, key);
  return (int)cudaGetLastError();
}

}  // namespace

#ifdef SG_CS_F32_UNIT
namespace sgcs {
int f32_stage(const CsParams& P, size_t faces, size_t cells, cudaStream_t s) {
  return launch_stage<float>(P, faces, cells, s);
}
int f32_ghost(const CsParams& P, void* buf, cudaStream_t s) {
  return launch_ghost<float>(P, buf, s);
}
int f32_dt(const CsParams& P, const void* buf, unsigned long long* key, int g,
           cudaStream_t s) {
  return launch_dt<float>(P, buf, key, g, s);
}
}  // namespace sgcs
#else

__global__ void to_f32(const double* src, float* dst, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}

struct sg_cs_handle {
  sg_cs_desc d;
  // SG_F32: FP32 copies of the geometry and of the two seam tables
  float* geo32 = nullptr;
  float* gtab32 = nullptr;
  float* stab32 = nullptr;
  float* sst32 = nullptr;
  void* buf[3] = {nullptr, nullptr, nullptr};
  void* scratch = nullptr;
  int cur = 0, base = 0;
  unsigned long long* key = nullptr;
  double* s2 = nullptr;  // the step fields (FP64, caller's memory)
  double* s3 = nullptr;
};

extern "C" {

int sg_cs_create(const sg_cs_desc* d, sg_cs_handle** out) {
  if (!d || !out) return cs_fail(SG_ERR_ARG, "sg_cs_create: null argument");
  *out = nullptr;
  if (d->n < 4 || d->ng != kNg)
    return cs_fail(SG_ERR_ARG, "sg_cs_create: n %d (>= 4), nghost %d (3)", d->n, d->ng);
  if (d->dtype != SG_F64 && d->dtype != SG_F32)
    return cs_fail(SG_ERR_ARG, "sg_cs_create: dtype %d", d->dtype);
  if (!d->geo || !d->ghost_tab || !d->seam_tab || d->nghost <= 0 || d->nseam <= 0)
    return cs_fail(SG_ERR_ARG, "sg_cs_create: the geometry and seam tables are required");
  if (d->riemann != SG_CS_SHALLOW_ROE && d->riemann != SG_CS_HLLC)
    return cs_fail(SG_ERR_ARG, "sg_cs_create: riemann %d", d->riemann);
  if (d->nstage < 1 || d->nstage > 3)
    return cs_fail(SG_ERR_ARG, "sg_cs_create: nstage %d", d->nstage);
  if (!d->seam_state_tab || d->nseam_state != 24 * d->n)
    return cs_fail(SG_ERR_ARG, "sg_cs_create: the seam face-state table needs "
                   "24 n = %d rows (got %d)", 24 * d->n, d->nseam_state);
  auto* h = new sg_cs_handle();
  h->d = *d;
  // key[0]: the min key, key[1]: a NaN flag
  cudaError_t e = cudaMalloc(&h->key, 2 * sizeof(unsigned long long));
  if (e == cudaSuccess) {
    const unsigned long long init[2] = {kKeyInf, 0};
    e = cudaMemcpy(h->key, init, sizeof(init), cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess && d->dtype == SG_F32) {
    // the FP32 kernels read FP32 copies; the tables' flat indices (cells,
    // and faces up to 6 nc (nc + 1)) stay exact in FP32 below 2^24
    const size_t nc = (size_t)d->n + 2 * kNg;
    if (6 * nc * (nc + 1) >= (size_t)1 << 24) {
      cudaFree(h->key);
      delete h;
      return cs_fail(SG_ERR_UNSUPPORTED, "sg_cs_create: FP32 needs fewer than "
                     "2^24 faces in the six panels (n %d)", d->n);
    }
    const size_t ng = 7 * nc * nc + 6 * nc * (nc + 1);
    const size_t nt = (size_t)kGhostStride * d->nghost;
    const size_t ns = (size_t)kSeamStride * d->nseam;
    const size_t nss = (size_t)kSeamStateStride * d->nseam_state;
    e = cudaMalloc(&h->geo32, ng * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&h->gtab32, nt * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&h->stab32, ns * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&h->sst32, nss * sizeof(float));
    if (e == cudaSuccess) {
      to_f32<<<grid_for(ng), kThreads>>>(d->geo, h->geo32, ng);
      to_f32<<<grid_for(nt), kThreads>>>(d->ghost_tab, h->gtab32, nt);
      to_f32<<<grid_for(ns), kThreads>>>(d->seam_tab, h->stab32, ns);
      to_f32<<<grid_for(nss), kThreads>>>(d->seam_state_tab, h->sst32, nss);
      e = cudaGetLastError();
      if (e == cudaSuccess) e = cudaDeviceSynchronize();
    }
  }
  if (e != cudaSuccess) {
    if (h->key) cudaFree(h->key);
    cudaFree(h->geo32);
    cudaFree(h->gtab32);
    cudaFree(h->stab32);
    cudaFree(h->sst32);
    delete h;
    return cs_fail(SG_ERR_CUDA, "sg_cs_create: %s", cudaGetErrorString(e));
  }
  *out = h;
  return 0;
}

int sg_cs_destroy(sg_cs_handle* h) {
  if (!h) return 0;
  if (h->key) cudaFree(h->key);
  cudaFree(h->geo32);
  cudaFree(h->gtab32);
  cudaFree(h->stab32);
  cudaFree(h->sst32);
  delete h;
  return 0;
}

int sg_cs_scratch_bytes(const sg_cs_handle* h, size_t* bytes) {
  if (!h || !bytes) return cs_fail(SG_ERR_ARG, "sg_cs_scratch_bytes: null");
  const size_t nc = (size_t)h->d.n + 2 * kNg;
  const size_t s = h->d.dtype == SG_F64 ? 8 : 4;
  // F2 and F3, then the seam faces' interior-side states
  *bytes = 2 * 6 * 4 * nc * (nc + 1) * s + 24 * (size_t)h->d.n * 4 * s;
  return 0;
}

int sg_cs_bind(sg_cs_handle* h, void* b0, void* b1, void* b2, void* scratch,
               size_t bytes) {
  size_t need = 0;
  if (!h) return cs_fail(SG_ERR_ARG, "sg_cs_bind: null handle");
  sg_cs_scratch_bytes(h, &need);
  if (!b0 || !b1 || !b2 || b0 == b1 || b1 == b2 || b0 == b2)
    return cs_fail(SG_ERR_ARG, "sg_cs_bind: three distinct non-null buffers needed");
  if (!scratch || bytes < need)
    return cs_fail(SG_ERR_ARG, "sg_cs_bind: the flux scratch needs %zu bytes", need);
  h->buf[0] = b0, h->buf[1] = b1, h->buf[2] = b2;
  h->scratch = scratch;
  return 0;
}

int sg_cs_set_current(sg_cs_handle* h, int32_t cur) {
  if (!h || cur < 0 || cur > 2) return cs_fail(SG_ERR_ARG, "sg_cs_set_current: %d", cur);
  h->cur = h->base = cur;
  return 0;
}

int sg_cs_rotation(const sg_cs_handle* h, int32_t* cur, int32_t* base) {
  if (!h || !cur || !base) return cs_fail(SG_ERR_ARG, "sg_cs_rotation: null");
  *cur = h->cur;
  *base = h->base;
  return 0;
}

int sg_cs_set_rotation(sg_cs_handle* h, int32_t cur, int32_t base) {
  if (!h || cur < 0 || cur > 2 || base < 0 || base > 2)
    return cs_fail(SG_ERR_ARG, "sg_cs_set_rotation: %d %d", cur, base);
  h->cur = cur;
  h->base = base;
  return 0;
}

static void cs_plan(const sg_cs_handle* h, int stage, int* in, int* u0, int* out) {
  *in = h->cur;
  *u0 = stage == 0 ? h->cur : h->base;
  int o = 0;
  while (o == *in || o == *u0) ++o;
  *out = o;
}

int sg_cs_advance(sg_cs_handle* h, int32_t stage) {
  if (!h || stage < 0 || stage >= h->d.nstage)
    return cs_fail(SG_ERR_ARG, "sg_cs_advance: stage %d", stage);
  int in, u0, out;
  cs_plan(h, stage, &in, &u0, &out);
  if (stage == 0) h->base = h->cur;
  h->cur = out;
  return 0;
}

static CsParams cs_params(const sg_cs_handle* h) {
  CsParams P = {};
  P.n = h->d.n;
  P.nc = h->d.n + 2 * kNg;
  const bool f32 = h->d.dtype == SG_F32;
  P.geo = f32 ? (const void*)h->geo32 : (const void*)h->d.geo;
  P.gtab = f32 ? (const void*)h->gtab32 : (const void*)h->d.ghost_tab;
  P.nghost = h->d.nghost;
  P.stab = f32 ? (const void*)h->stab32 : (const void*)h->d.seam_tab;
  P.nseam = h->d.nseam;
  P.sst = f32 ? (const void*)h->sst32 : (const void*)h->d.seam_state_tab;
  P.phi0 = h->d.dtype == SG_F32 ? h->d.phi_ref : 0.;
  P.hllc = h->d.riemann == SG_CS_HLLC;
  const size_t nc = P.nc;
  const size_t s = h->d.dtype == SG_F64 ? 8 : 4;
  P.s2 = h->s2;
  P.s3 = h->s3;
  P.geo64 = h->d.geo;
  P.f2 = h->scratch;
  P.f3 = static_cast<unsigned char*>(h->scratch) + 6 * 4 * nc * (nc + 1) * s;
  P.sbuf = static_cast<unsigned char*>(h->scratch) + 2 * 6 * 4 * nc * (nc + 1) * s;
  return P;
}

int sg_cs_fill_seams(sg_cs_handle* h, sg_stream_t stream) {
  if (!h || !h->buf[0]) return cs_fail(SG_ERR_STATE, "sg_cs_fill_seams: buffers not bound");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  CsParams P = cs_params(h);
  const int rc = h->d.dtype == SG_F64 ? launch_ghost<double>(P, h->buf[h->cur], s)
                                      : sgcs::f32_ghost(P, h->buf[h->cur], s);
  cudaError_t e = rc ? (cudaError_t)rc : cudaGetLastError();
  return e == cudaSuccess ? 0 : cs_fail(SG_ERR_CUDA, "sg_cs_fill_seams: %s", cudaGetErrorString(e));
}

int sg_cs_stage(sg_cs_handle* h, int32_t stage, const double* dt_dev,
                sg_stream_t stream) {
  if (!h || !dt_dev) return cs_fail(SG_ERR_ARG, "sg_cs_stage: null argument");
  if (!h->buf[0]) return cs_fail(SG_ERR_STATE, "sg_cs_stage: buffers not bound");
  if (stage < 0 || stage >= h->d.nstage)
    return cs_fail(SG_ERR_ARG, "sg_cs_stage: stage %d of %d", stage, h->d.nstage);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int in, u0, out;
  cs_plan(h, stage, &in, &u0, &out);
  CsParams P = cs_params(h);
  P.in = h->buf[in];
  P.u0 = h->buf[u0];
  P.out = h->buf[out];
  P.dt = dt_dev;
  P.w0 = h->d.wght[stage][0];
  P.w1 = h->d.wght[stage][1];
  P.w2 = h->d.wght[stage][2];
  P.first = stage == 0;
  const size_t faces = (size_t)2 * 6 * P.n * (P.n + 1);
  const size_t cells = (size_t)6 * P.n * P.n;
  const int rc = h->d.dtype == SG_F64 ? launch_stage<double>(P, faces, cells, s)
                                      : sgcs::f32_stage(P, faces, cells, s);
  cudaError_t e = rc ? (cudaError_t)rc : cudaGetLastError();
  if (e != cudaSuccess) return cs_fail(SG_ERR_CUDA, "sg_cs_stage: %s", cudaGetErrorString(e));
  if (stage == 0) h->base = h->cur;
  h->cur = out;
  return 0;
}

int sg_cs_bind_step_fields(sg_cs_handle* h, double* s2, double* s3) {
  if (!h) return cs_fail(SG_ERR_ARG, "sg_cs_bind_step_fields: null handle");
  if ((s2 == nullptr) != (s3 == nullptr))
    return cs_fail(SG_ERR_ARG, "sg_cs_bind_step_fields: both fields or neither");
  h->s2 = s2;
  h->s3 = s3;
  return 0;
}

int sg_cs_budget_totals(sg_cs_handle* h, double* out, sg_stream_t stream) {
  if (!h || !out) return cs_fail(SG_ERR_ARG, "sg_cs_budget_totals: null argument");
  if (!h->buf[0]) return cs_fail(SG_ERR_STATE, "sg_cs_budget_totals: buffers not bound");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  CsParams P = cs_params(h);
  if (h->d.dtype == SG_F64)
    cs_budget_kernel<double><<<1, kBudgetThreads, 0, s>>>(P, h->buf[h->cur], out);
  else
    cs_budget_kernel<float><<<1, kBudgetThreads, 0, s>>>(P, h->buf[h->cur], out);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : cs_fail(SG_ERR_CUDA, "sg_cs_budget_totals: %s", cudaGetErrorString(e));
}

int sg_cs_max_dt(sg_cs_handle* h, double* dt_dev, sg_stream_t stream) {
  if (!h || !dt_dev) return cs_fail(SG_ERR_ARG, "sg_cs_max_dt: null argument");
  if (!h->buf[0]) return cs_fail(SG_ERR_STATE, "sg_cs_max_dt: buffers not bound");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  CsParams P = cs_params(h);
  const size_t cells = (size_t)6 * P.n * P.n;
  int g = grid_for(cells);
  if (g > 256) g = 256;
  if (h->d.dtype == SG_F64)
    launch_dt<double>(P, h->buf[h->cur], h->key, g, s);
  else
    sgcs::f32_dt(P, h->buf[h->cur], h->key, g, s);
  cs_dt_finish<<<1, 1, 0, s>>>(h->key, h->d.cfl, dt_dev);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : cs_fail(SG_ERR_CUDA, "sg_cs_max_dt: %s", cudaGetErrorString(e));
}

}  // extern "C"

#endif  // SG_CS_F32_UNIT
