// Device arithmetic of the hydro stage: reconstruction, Riemann face fluxes
// and the ideal-gas EOS, templated on the compute type T.
//
// Each function keeps the reference's order of floating-point operations so
// that the FP64 instantiation (compiled with -fmad=false) reproduces the
// reference CPU path bit for bit at every face:
//   weno5_cm / weno5_cp  src/recon/recon_point.h:114-147 with the uniform
//                        tables of src/recon/reconstruct.cpp:71-88, terms with
//                        a zero coefficient dropped (x + 0 == x)
//   cp5_cm / cp5_cp      src/recon/recon_point.h:53-61, reconstruct.cpp:63-68
//   hllc_flux            src/riemann/riemann_kernels.h:56-194
//   lmars_flux           src/riemann/riemann_kernels.h:197-255
//   cons2prim            src/eos/ideal_gas_impl.h:16-35
#pragma once

#include <cuda_runtime.h>
#include <math.h>

namespace sg {

enum { IDN = 0, IVX = 1, IVY = 2, IVZ = 3, IPR = 4, NHYDRO = 5 };

// a float widened to the double of the same value with integer operations
// only: the FP64 kernels here are bound by the FP64 pipe, which the widening
// instruction would also occupy.  Normal numbers rebias the exponent (127 ->
// 1023) and shift the mantissa up 29 bits; zeros keep their sign; a
// subnormal m 2^-149 is renormalised at its leading bit; infinities and NaNs
// keep their payload (the quiet bit lands on the double's)
__device__ __forceinline__ unsigned long long widen_bits(unsigned int b) {
  const unsigned long long sgn = (unsigned long long)(b >> 31) << 63;
  const unsigned int e = (b >> 23) & 0xffu;
  const unsigned long long m = b & 0x7fffffu;
  if (e == 0xffu) return sgn | (0x7ffull << 52) | (m << 29);
  if (e != 0u) return sgn | ((unsigned long long)(e + 896u) << 52) | (m << 29);
  if (m == 0u) return sgn;
  const int k = 31 - __clz((int)m);  // the leading bit, 0..22
  return sgn | ((unsigned long long)(k + 874) << 52) |
         ((m << (52 - k)) & 0xfffffffffffffull);
}

__device__ __forceinline__ double widen_exact(float f) {
  return __longlong_as_double((long long)widen_bits(__float_as_uint(f)));
}

// a double rounded to the nearest float (ties to even) with integer
// operations only, for the same reason: the conversion instruction runs on
// the FP64 pipe.  Overflow gives infinity, results below the normal range
// are rounded to float subnormals (or zero), NaNs stay NaNs (quiet, the
// payload's top bits kept)
__device__ __forceinline__ unsigned int narrow_bits(unsigned long long d) {
  const unsigned int sgn = (unsigned int)(d >> 63) << 31;
  const int e = (int)((d >> 52) & 0x7ff);
  const unsigned long long m = d & 0xfffffffffffffull;
  if (e == 0x7ff)
    return sgn | 0x7f800000u | (m ? (0x400000u | (unsigned int)(m >> 29)) : 0u);
  int ef = e - 1023 + 127;  // the float's biased exponent
  if (ef >= 255) return sgn | 0x7f800000u;
  const unsigned long long M = m | (e ? (1ull << 52) : 0ull);
  int sh = 29;  // the bits a normal float drops
  if (ef <= 0) {  // a float subnormal, or zero
    sh = 30 - ef;
    if (sh > 54) return sgn;
    ef = 0;
  }
  unsigned long long keep = M >> sh;
  const unsigned long long rem = M & ((1ull << sh) - 1), half = 1ull << (sh - 1);
  if (rem > half || (rem == half && (keep & 1))) keep += 1;
  // a normal keeps its implicit bit at 23; a carry out of the mantissa bumps
  // the exponent (254 -> infinity)
  return sgn | (ef ? ((unsigned int)ef << 23) + (unsigned int)(keep - (1ull << 23))
                   : (unsigned int)keep);
}

__device__ __forceinline__ float narrow_exact(double x) {
  return __uint_as_float(narrow_bits((unsigned long long)__double_as_longlong(x)));
}

// a double in the storage type (to a float through the integer pipes)
template <typename T>
__device__ __forceinline__ T as_real(double x);
template <>
__device__ __forceinline__ double as_real<double>(double x) { return x; }
template <>
__device__ __forceinline__ float as_real<float>(double x) { return narrow_exact(x); }

// a value of the storage type in FP64 (a float through the integer pipes)
__device__ __forceinline__ double as_f64(double x) { return x; }
__device__ __forceinline__ double as_f64(float x) { return widen_exact(x); }

template <typename T>
__device__ __forceinline__ T sqr(T x) {
  return x * x;
}

// a / b from r = 1 / b (the correctly rounded reciprocal): q0 = a r, the
// exact residual a - b q0 by one fma, then q0 + e r rounded once.  For
// normal operands and quotient this is the correctly rounded quotient, the
// same bits as a / b (Markstein, "Computation of elementary functions on
// the IBM RISC System/6000 processor", IBM J. Res. Dev. 34 (1990), and
// "IA-64 and Elementary Functions" (2000), the division theorem); it costs
// one multiply and two fmas where a division is a longer sequence, and the
// reciprocal is shared by every quotient with the same divisor
template <typename T>
__device__ __forceinline__ T vdiv(T a, T b, T r) {
  const T q0 = a * r;
  const T e = fma(-b, q0, a);
  return fma(e, r, q0);
}


// exp(x) for the well-balanced reference's anchor, written out so that the
// GPU kernel and the CPU oracle evaluate the same operations and agree bit
// for bit (libm's and CUDA's exp may differ by an ulp, which the anchor
// turns into a 1e-12 difference of small pressure perturbations).  Method:
// Cody-Waite argument reduction x = k ln2 + r, |r| <= ln2/2, with ln2 split
// into a 32-bit head and a tail, then the Taylor series of exp(r) to r^16
// in Horner form, scaled by 2^k.  Accurate to about 2 ulp for |x| < 700.
__device__ __forceinline__ double sg_exp(double x) {
  const double ln2_hi = 6.93147180369123816490e-01;  // 0x3fe62e42fee00000
  const double ln2_lo = 1.90821492927058770002e-10;
  const double inv_ln2 = 1.44269504088896338700e+00;
  double k = rint(x * inv_ln2);
  double r = (x - k * ln2_hi) - k * ln2_lo;
  double p = 1.0 / 20922789888000.0;  // 1/16!
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

// WENO5 with the cm table: the state on the +side of the LOWER face of the
// centre cell f2 (phi = f0..f4 = cells c-2..c+2). scale: InterpOptions::scale.
template <typename T>
__device__ __forceinline__ T weno5_cm(T f0, T f1, T f2, T f3, T f4,
                                      bool scale) {
  T vscale = T(1.0);
  if (scale) {
    T sum = fabs(f0);
    sum += fabs(f1);
    sum += fabs(f2);
    sum += fabs(f3);
    sum += fabs(f4);
    vscale = sum / T(5);
    if (vscale == T(0)) return T(0);
    f0 = f0 / vscale, f1 = f1 / vscale, f2 = f2 / vscale, f3 = f3 / vscale,
    f4 = f4 / vscale;
  }
  T p0 = (T(-1. / 6.) * f0 + T(5. / 6.) * f1) + T(1. / 3.) * f2;
  T p1 = (T(1. / 3.) * f1 + T(5. / 6.) * f2) + T(-1. / 6.) * f3;
  T p2 = (T(11. / 6.) * f2 + T(-7. / 6.) * f3) + T(1. / 3.) * f4;
  T a = (f0 + T(-2.) * f1) + f2;
  T b = (f0 + T(-4.) * f1) + T(3.) * f2;
  T beta0 = T(13. / 12.) * (a * a) + T(.25) * (b * b);
  a = (f1 + T(-2.) * f2) + f3;
  b = -f1 + f3;
  T beta1 = T(13. / 12.) * (a * a) + T(.25) * (b * b);
  a = (f2 + T(-2.) * f3) + f4;
  b = (T(3.) * f2 + T(-4.) * f3) + f4;
  T beta2 = T(13. / 12.) * (a * a) + T(.25) * (b * b);
  const T eps = T(1e-6);
  T alpha0 = T(.3) / sqr(beta0 + eps);
  T alpha1 = T(.6) / sqr(beta1 + eps);
  T alpha2 = T(.1) / sqr(beta2 + eps);
  return vscale * (alpha0 * p0 + alpha1 * p1 + alpha2 * p2) /
         (alpha0 + alpha1 + alpha2);
}

// WENO5 with the cp table (each row reversed): the state on the -side of the
// UPPER face of the centre cell f2.
template <typename T>
__device__ __forceinline__ T weno5_cp(T f0, T f1, T f2, T f3, T f4,
                                      bool scale) {
  T vscale = T(1.0);
  if (scale) {
    T sum = fabs(f0);
    sum += fabs(f1);
    sum += fabs(f2);
    sum += fabs(f3);
    sum += fabs(f4);
    vscale = sum / T(5);
    if (vscale == T(0)) return T(0);
    f0 = f0 / vscale, f1 = f1 / vscale, f2 = f2 / vscale, f3 = f3 / vscale,
    f4 = f4 / vscale;
  }
  T p0 = (T(1. / 3.) * f2 + T(5. / 6.) * f3) + T(-1. / 6.) * f4;
  T p1 = (T(-1. / 6.) * f1 + T(5. / 6.) * f2) + T(1. / 3.) * f3;
  T p2 = (T(1. / 3.) * f0 + T(-7. / 6.) * f1) + T(11. / 6.) * f2;
  T a = (f2 + T(-2.) * f3) + f4;
  T b = (T(3.) * f2 + T(-4.) * f3) + f4;
  T beta0 = T(13. / 12.) * (a * a) + T(.25) * (b * b);
  a = (f1 + T(-2.) * f2) + f3;
  b = f1 + -f3;
  T beta1 = T(13. / 12.) * (a * a) + T(.25) * (b * b);
  a = (f0 + T(-2.) * f1) + f2;
  b = (f0 + T(-4.) * f1) + T(3.) * f2;
  T beta2 = T(13. / 12.) * (a * a) + T(.25) * (b * b);
  const T eps = T(1e-6);
  T alpha0 = T(.3) / sqr(beta0 + eps);
  T alpha1 = T(.6) / sqr(beta1 + eps);
  T alpha2 = T(.1) / sqr(beta2 + eps);
  return vscale * (alpha0 * p0 + alpha1 * p1 + alpha2 * p2) /
         (alpha0 + alpha1 + alpha2);
}

template <typename T>
__device__ __forceinline__ T cp5_cm(T f0, T f1, T f2, T f3, T f4) {
  return (((T(-1. / 20.) * f0 + T(9. / 20.) * f1) + T(47. / 60.) * f2) +
          T(-13. / 60.) * f3) +
         T(1. / 30.) * f4;
}

template <typename T>
__device__ __forceinline__ T cp5_cp(T f0, T f1, T f2, T f3, T f4) {
  return (((T(1. / 30.) * f0 + T(-13. / 60.) * f1) + T(47. / 60.) * f2) +
          T(9. / 20.) * f3) +
         T(-1. / 20.) * f4;
}

// the face-normal and the two tangential velocity rows of a face whose
// normal is x<d> (d = 1, 2, 3), riemann_kernels.h:34-38
struct Axes {
  int x, y, z;
};
__device__ __forceinline__ Axes face_axes(int d) {
  int ivx = IVX + d - 1;
  return {ivx, IVX + ((ivx - IVX) + 1) % 3, IVX + ((ivx - IVX) + 2) % 3};
}

// HLLC face flux, ideal gas (e = p/(g-1), c = sqrt(g p / rho)), no species
template <typename T>
__device__ __forceinline__ void hllc_flux(const T* wl, const T* wr, T gammad,
                                          int d, T* flx, T* face_pressure) {
  Axes ax = face_axes(d);
  const int ivx = ax.x, ivy = ax.y, ivz = ax.z;
  T el = wl[IPR] / (gammad - T(1));
  T er = wr[IPR] / (gammad - T(1));
  T cl = sqrt(gammad * wl[IPR] / wl[IDN]);
  T cr = sqrt(gammad * wr[IPR] / wr[IDN]);
  T pl = wl[IPR], pr = wr[IPR];

  el += T(0.5) * wl[IDN] * (sqr(wl[IVX]) + sqr(wl[IVY]) + sqr(wl[IVZ]));
  er += T(0.5) * wr[IDN] * (sqr(wr[IVX]) + sqr(wr[IVY]) + sqr(wr[IVZ]));

  T rhoa = T(0.5) * (wl[IDN] + wr[IDN]);
  T ca = T(0.5) * (cl + cr);
  T pmid = T(0.5) * (wl[IPR] + wr[IPR] + (wl[ivx] - wr[ivx]) * rhoa * ca);

  T shock_l = pmid / wl[IPR] - T(1.0);
  T shock_r = pmid / wr[IPR] - T(1.0);
  T ql = (pmid <= wl[IPR])
             ? T(1.0)
             : sqrt(T(1.0) + (gammad + T(1)) / (T(2) * gammad) * shock_l);
  T qr = (pmid <= wr[IPR])
             ? T(1.0)
             : sqrt(T(1.0) + (gammad + T(1)) / (T(2) * gammad) * shock_r);

  T al = wl[ivx] - cl * ql;
  T ar = wr[ivx] + cr * qr;
  T bp = ar > T(0.0) ? ar : T(1.0e-10);
  T bm = al < T(0.0) ? al : -T(1.0e-10);

  T vxl, vxr;
  if (sizeof(T) == 4) {  // riemann_kernels.h:99-105, the float branch
    vxl = cl * ql;
    vxr = -cr * qr;
  } else {
    vxl = wl[ivx] - al;
    vxr = wr[ivx] - ar;
  }
  T tl = wl[IPR] + vxl * wl[IDN] * wl[ivx];
  T tr = wr[IPR] + vxr * wr[IDN] * wr[ivx];
  T ml = wl[IDN] * vxl;
  T mr = -(wr[IDN] * vxr);
  T am = (tl - tr) / (ml + mr);
  T cp = (ml * tr + mr * tl) / (ml + mr);
  cp = cp > T(0.0) ? cp : T(0.0);
  if (face_pressure) *face_pressure = cp;

  if (sizeof(T) == 4) {
    vxl = al < T(0) ? cl * ql : wl[ivx] + T(1.0e-10);
    vxr = ar > T(0) ? -cr * qr : wr[ivx] - T(1.0e-10);
  } else {
    vxl = wl[ivx] - bm;
    vxr = wr[ivx] - bp;
  }
  T fl[5], fr[5];
  fl[IDN] = wl[IDN] * vxl;
  fr[IDN] = wr[IDN] * vxr;
  fl[ivx] = wl[IDN] * wl[ivx] * vxl + wl[IPR];
  fr[ivx] = wr[IDN] * wr[ivx] * vxr + wr[IPR];
  fl[ivy] = wl[IDN] * wl[ivy] * vxl;
  fr[ivy] = wr[IDN] * wr[ivy] * vxr;
  fl[ivz] = wl[IDN] * wl[ivz] * vxl;
  fr[ivz] = wr[IDN] * wr[ivz] * vxr;
  fl[IPR] = el * vxl + pl * wl[ivx];
  fr[IPR] = er * vxr + pr * wr[ivx];

  T sl, sr, sm;
  if (am >= T(0.0)) {
    sl = am / (am - bm);
    sr = T(0.0);
    sm = -bm / (am - bm);
  } else {
    sl = T(0.0);
    sr = -am / (bp - am);
    sm = bp / (bp - am);
  }
  flx[IDN] = sl * fl[IDN] + sr * fr[IDN];
  flx[ivx] = sl * fl[ivx] + sr * fr[ivx] + sm * cp;
  flx[ivy] = sl * fl[ivy] + sr * fr[ivy];
  flx[ivz] = sl * fl[ivz] + sr * fr[ivz];
  flx[IPR] = sl * fl[IPR] + sr * fr[IPR] + sm * cp * am;
}

// LMARS face flux, ideal gas (h = p/(g-1)/rho + ...), no species
template <typename T>
__device__ __forceinline__ void lmars_flux(const T* wl, const T* wr, T gammad,
                                           int d, T* flx, T* face_pressure) {
  Axes ax = face_axes(d);
  const int ivx = ax.x, ivy = ax.y, ivz = ax.z;
  // the quotients by gamma - 1 and by each side's density divide through
  // the reciprocals (vdiv: the same bits)
  const T gm1 = gammad - T(1), rgm1 = T(1) / gm1;
  const T rl0 = T(1) / wl[IDN], rr0 = T(1) / wr[IDN];
  T hl = vdiv(vdiv(wl[IPR], gm1, rgm1), wl[IDN], rl0);
  T hr = vdiv(vdiv(wr[IPR], gm1, rgm1), wr[IDN], rr0);
  T l0 = wl[IDN], l1 = wl[ivx], l2 = wl[ivy], l3 = wl[ivz], l4 = wl[IPR];
  T r0 = wr[IDN], r1 = wr[ivx], r2 = wr[ivy], r3 = wr[ivz], r4 = wr[IPR];
  hl += T(0.5) * (sqr(l1) + sqr(l2) + sqr(l3)) + vdiv(l4, l0, rl0);
  hr += T(0.5) * (sqr(r1) + sqr(r2) + sqr(r3)) + vdiv(r4, r0, rr0);
  T rhobar = T(0.5) * (l0 + r0);
  T gamma_bar = T(0.5) * (gammad + gammad);
  T cbar = sqrt(T(0.5) * gamma_bar * (l4 + r4) / rhobar);
  T pbar = T(0.5) * (l4 + r4) + T(0.5) * (rhobar * cbar) * (l1 - r1);
  if (face_pressure) *face_pressure = pbar;
  T ubar = T(0.5) * (l1 + r1) + T(0.5) / (rhobar * cbar) * (l4 - r4);
  if (ubar > T(0)) {
    flx[IDN] = ubar * l0;
    flx[ivx] = ubar * l0 * l1 + pbar;
    flx[ivy] = ubar * l0 * l2;
    flx[ivz] = ubar * l0 * l3;
    flx[IPR] = ubar * l0 * hl;
  } else {
    flx[IDN] = ubar * r0;
    flx[ivx] = ubar * r0 * r1 + pbar;
    flx[ivy] = ubar * r0 * r2;
    flx[ivz] = ubar * r0 * r3;
    flx[IPR] = ubar * r0 * hr;
  }
}

// LMARS on pressure ANOMALIES: wl[IPR], wr[IPR] are p - pb, with pb the
// base pressure at the face (the same on both sides).  The totals give the
// sound speed and the enthalpy; the face pressure is affine in (pl, pr)
// with weights summing to one, so the momentum flux carries pbar - pb and
// the base's share (pb itself) is left to the caller's hydrostatic balance.
// Used by the FP32 state, whose pressure only has the precision of an
// anomaly.
template <typename T>
__device__ __forceinline__ void lmars_flux_anom(const T* wl, const T* wr,
                                                T gammad, int d, T pb,
                                                T* flx) {
  Axes ax = face_axes(d);
  const int ivx = ax.x, ivy = ax.y, ivz = ax.z;
  T l0 = wl[IDN], l1 = wl[ivx], l2 = wl[ivy], l3 = wl[ivz], l4 = wl[IPR];
  T r0 = wr[IDN], r1 = wr[ivx], r2 = wr[ivy], r3 = wr[ivz], r4 = wr[IPR];
  T pl = pb + l4, pr = pb + r4;
  const T gm1 = gammad - T(1), rgm1 = T(1) / gm1;
  const T rl0 = T(1) / l0, rr0 = T(1) / r0;
  T hl = vdiv(vdiv(pl, gm1, rgm1), l0, rl0);
  T hr = vdiv(vdiv(pr, gm1, rgm1), r0, rr0);
  hl += T(0.5) * (sqr(l1) + sqr(l2) + sqr(l3)) + vdiv(pl, l0, rl0);
  hr += T(0.5) * (sqr(r1) + sqr(r2) + sqr(r3)) + vdiv(pr, r0, rr0);
  T rhobar = T(0.5) * (l0 + r0);
  T cbar = sqrt(T(0.5) * gammad * (pl + pr) / rhobar);
  T pbar = T(0.5) * (l4 + r4) + T(0.5) * (rhobar * cbar) * (l1 - r1);
  T ubar = T(0.5) * (l1 + r1) + T(0.5) / (rhobar * cbar) * (l4 - r4);
  const T m0 = ubar > T(0) ? l0 : r0;
  const T v1 = ubar > T(0) ? l1 : r1, v2 = ubar > T(0) ? l2 : r2,
          v3 = ubar > T(0) ? l3 : r3, h = ubar > T(0) ? hl : hr;
  flx[IDN] = ubar * m0;
  flx[ivx] = ubar * m0 * v1 + pbar;
  flx[ivy] = ubar * m0 * v2;
  flx[ivz] = ubar * m0 * v3;
  flx[IPR] = ubar * m0 * h;
}

// ideal-gas U->W of one cell (Cartesian: the metric raise is the identity);
// the three velocities divide by the density through its reciprocal (vdiv:
// the same quotients)
template <typename T>
__device__ __forceinline__ void cons2prim(const T* u, T* w, T gammad) {
  w[IDN] = u[IDN];
  const T rd = T(1.) / w[IDN];
  w[IVX] = vdiv(u[IVX], w[IDN], rd);
  w[IVY] = vdiv(u[IVY], w[IDN], rd);
  w[IVZ] = vdiv(u[IVZ], w[IDN], rd);
  T ke = T(0.5) * (w[IVX] * u[IVX] + w[IVY] * u[IVY] + w[IVZ] * u[IVZ]);
  T ie = u[IPR] - ke;
  w[IPR] = (gammad - T(1.)) * ie;
}

}  // namespace sg
