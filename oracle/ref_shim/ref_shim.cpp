// Thin extern "C" wrappers around the reference's own header-only face
// kernels, compiled unmodified from the reference source tree by
// oracle/Makefile into oracle/_ref/libsnapref.so.  TEST INFRASTRUCTURE ONLY:
// the oracle's restatement (oracle/sg_oracle.c) is checked against these in
// tests/test_oracle_pin.py.  Nothing here is shipped or timed as the product.
//
// Headers compiled: src/recon/recon_point.h, src/riemann/riemann_kernels.h,
// src/eos/ideal_gas_impl.h, src/hydro/hydro_ref_x1_impl.h.
#include <snap/recon/recon_point.h>
#include <snap/riemann/riemann_kernels.h>
#include <snap/eos/ideal_gas_impl.h>
#include <snap/hydro/hydro_ref_x1_impl.h>

namespace {
// the uniform tables of reconstruct.cpp:49-93 (InterpImpl::reset): nine
// stencil rows then d for weno5; cp = each row reversed
const double kRows[9][5] = {
    {-1. / 6., 5. / 6., 1. / 3., 0., 0.}, {0., 1. / 3., 5. / 6., -1. / 6., 0.},
    {0., 0., 11. / 6., -7. / 6., 1. / 3.}, {1., -2., 1., 0., 0.},
    {1., -4., 3., 0., 0.},                  {0., 1., -2., 1., 0.},
    {0., -1., 0., 1., 0.},                  {0., 0., 1., -2., 1.},
    {0., 0., 3., -4., 1.}};
const double kD[3] = {.3, .6, .1};
const double kCp5[5] = {-1. / 20., 9. / 20., 47. / 60., -13. / 60., 1. / 30.};

void table(int side, double* t) {
  for (int r = 0; r < 9; ++r)
    for (int k = 0; k < 5; ++k) t[r * 5 + k] = side ? kRows[r][4 - k] : kRows[r][k];
  for (int k = 0; k < 3; ++k) t[45 + k] = kD[k];
}
}  // namespace

extern "C" {

double ref_weno5_point(const double* s5, int side, int scale) {
  double t[48];
  table(side, t);
  return snap::weno5_point<double>(s5, 1, t, scale != 0);
}

double ref_cp5_point(const double* s5, int side) {
  double c[5];
  for (int k = 0; k < 5; ++k) c[k] = side ? kCp5[4 - k] : kCp5[k];
  return snap::poly_point<double, 5>(s5, 1, c);
}

void ref_hllc(double* flx, double* wl, double* wr, double el, double er,
              double gl, double gr, double cl, double cr, int dim,
              double* face_pressure) {
  snap::hllc_impl<double>(flx, wl, wr, el, er, gl, gr, cl, cr, dim, 0, 1, 1,
                          face_pressure);
}

void ref_lmars(double* flx, double* wl, double* wr, double hl, double hr,
               double gl, double gr, int dim, double* face_pressure) {
  snap::lmars_impl<double>(flx, wl, wr, hl, hr, gl, gr, dim, 0, 1, 1,
                           face_pressure);
}

void ref_shallow_roe(double* flx, const double* wl, const double* wr, int dim,
                     int dir_yz) {
  snap::shallow_roe_impl<double>(flx, wl, wr, dim, dir_yz, 1, 1);
}

void ref_cons2prim(double* prim, double* cons, double gammad) {
  double cth = 0.;
  snap::ideal_gas_cons2prim<double>(prim, cons, &cth, gammad, 1);
}

// one column of the hydrostatic face-pressure scan (hydro_ref_x1_impl.h)
void ref_pressure_scan(const double* w, const double* dx1f, double* psf_lo,
                       double* psf_hi, int nc1, int iu, double grav) {
  snap::hydro_ref_x1_scan_impl<double>(w, dx1f, nullptr, psf_lo, psf_hi, 0, 1,
                                       nc1, iu, grav);
}

// the whole per-column reference of hydro_ref_x1_impl (scan, cell pressure,
// face and cell densities) on a uniform x1 grid, one column
void ref_hydro_ref_column(const double* w, const double* dx1f, double* psf_lo,
                          double* psf_hi, double* pref, double* dsf,
                          double* dref, int nc1, int iu, double grav,
                          int phys_in, int phys_out, int wall_clamp) {
  snap::hydro_ref_x1_impl<double>(w, dx1f, nullptr, psf_lo, psf_hi, pref, dsf,
                                  dref, 0, 1, nc1, iu, grav,
                                  snap::kX1RefUniform, phys_in != 0,
                                  phys_out != 0, wall_clamp != 0, nullptr);
}

}  // extern "C"
