"""CPU restatement of the cubed-sphere shallow-water stage (FP64): TEST
INFRASTRUCTURE ONLY -- the checker of the GPU path, never part of it.

The array plumbing is numpy; the pointwise reconstruction (WENO5 / cp5) and
the shallow-roe solver are the C oracle's (oracle/sg_oracle.c), pinned to the
reference's kernels.  The grid geometry and the panel-seam exchanges (the
ghost halo, the face states at the seams, the single-valued seam fluxes) are
oracle/cs_seams.py's restatement of the reference's own routines; nothing is
taken from the product's tables.

One stage follows the reference (src/hydro/hydro_forward.cpp with the
gnomonic coordinate of src/coord/gnomonic_equiangle.cpp):
  W = U/Phi with the momenta raised by the cell cosine (ShallowWaterImpl::
  _cons2prim, src/eos/shallow_water.cpp:30-42; coord_vec_raise_impl,
  src/coord/coord_utils_impl.h:9-16);
  x2 / x3 face states, weno5 for Phi and cp5 for the velocities
  (reconstruct.cpp:151-187), then the cross-panel face-state sync at the
  seams (hydro_forward.cpp:719-757, cs_seams.seam_states_all);
  to the face frame (prim2local2_/3_, gnomonic_equiangle.cpp:357-398),
  shallow_roe with dir yz (riemann_kernels.h:447-495) or the product's
  shallow-water HLLC (og_hllc_sw_batch, no reference counterpart), back to
  covariant fluxes (flux2global2_/3_, :414-463);
  the seam faces single-valued (reconcile_panel_seams, seam_register.cpp:35,
  cs_seams.reconcile);
  div = (A2 dF2 + A3 dF3) / V (coordinate.cpp:618-662), minus the metric
  sources x_ov_rD (p + Phi v3 v3 sin^2), y_ov_rC (p + Phi v2 v2 sin^2),
  p = Phi^2 / 2 (gnomonic_equiangle.cpp:465-521); du = -dt div;
  the RK combine, then the seam halo fill (cs_seams.fill).
With step fields requested, every stage also sets S_d <- w1 S_d + w2 dt T_d
over the stage's final (reconciled) face fluxes (FluxRegister::end_stage,
src/hydro/flux_register.hpp:241-402), S_d = 0 at stage 0; the budget's row
totals are sum u V over the interior (budget.cpp:68-200).
"""
from __future__ import annotations

import numpy as np

from . import cs_seams as R
from . import oracle as O

NG = 3
IDN, IVX, IVY, IVZ = 0, 1, 2, 3


def _recon(st: np.ndarray, weno: bool, side: int) -> np.ndarray:
    st = np.ascontiguousarray(st.reshape(-1, 5))
    out = np.zeros(st.shape[0])
    O.lib().og_recon_batch(O.ptr(st.ravel()), st.shape[0], int(weno), side, 0,
                           O.ptr(out))
    return out


def _roe(wl: np.ndarray, wr: np.ndarray, dim: int, hllc: bool = False) -> np.ndarray:
    wl = np.ascontiguousarray(wl.reshape(-1, 4))
    wr = np.ascontiguousarray(wr.reshape(-1, 4))
    f = np.zeros_like(wl)
    fn = O.lib().og_hllc_sw_batch if hllc else O.lib().og_shallow_roe_batch
    fn(O.ptr(wl.ravel()), O.ptr(wr.ravel()), wl.shape[0], dim, O.ptr(f.ravel()))
    return f


class CubedSphere:
    """Six panels (6, 4, nc, nc) FP64: Phi, and the radial and the two
    covariant tangential momenta, on the reference's geometry (radius r,
    one radial cell [r, r + 1] as examples/shallow_splash.yaml has it)."""

    def __init__(self, n, wght, cfl, riemann="shallow-roe", radius=6.371e6):
        self.n = n
        self.g = R.geometry(n, radius)
        self.hllc = riemann == "hllc"
        self.wght, self.cfl = wght, cfl
        self.nc = n + 2 * NG
        self.steps = None  # the step fields S_2, S_3, once requested

    def request_step_fields(self):
        nc = self.nc
        self.steps = {2: np.zeros((6, 4, nc, nc + 1)), 3: np.zeros((6, 4, nc + 1, nc))}
        return self.steps

    def budget_totals(self, u):
        I = slice(NG, NG + self.n)
        return (u[:, :, I, I] * self.g["vol"][I, I]).sum(axis=(0, 2, 3))

    def cons2prim(self, u):
        w = np.empty_like(u)
        w[:, IDN] = u[:, IDN]
        # the panels' corner ghosts are never filled (no stencil reads them)
        with np.errstate(divide="ignore", invalid="ignore"):
            v = u[:, IVX:IVZ + 1] / u[:, IDN:IDN + 1]
        c = self.g["cos_c"]
        sth2 = 1. - c * c
        w[:, IVX] = v[:, 0]
        w[:, IVY] = v[:, 1] / sth2 - v[:, 2] * c / sth2
        w[:, IVZ] = -v[:, 1] * c / sth2 + v[:, 2] / sth2
        return w

    def fill(self, u):
        """The seam halo of every panel (in place)."""
        R.fill(u, self.g)

    def _states(self, w, axis):
        """Face states of one direction: x2 (axis 2: faces j = NG..NG+n of
        rows k = NG..NG+n-1) or x3 (axis 1); (wl, wr) each (6, 4, ...)."""
        n = self.n
        fi = np.arange(NG, NG + n + 1)  # faces
        ri = np.arange(NG, NG + n)      # rows
        if axis == 2:
            st = np.stack([w[:, :, ri][:, :, :, fi + o] for o in range(-3, 3)], -1)
        else:
            st = np.stack([w[:, :, fi + o][:, :, :, ri] for o in range(-3, 3)], -1)
        wl = np.empty(st.shape[:-1])
        wr = np.empty(st.shape[:-1])
        for v in range(4):
            weno = v == IDN
            wl[:, v] = _recon(st[:, v, ..., 0:5], weno, 1).reshape(wl[:, v].shape)
            wr[:, v] = _recon(st[:, v, ..., 1:6], weno, 0).reshape(wr[:, v].shape)
        return wl, wr

    def _faces(self, wl, wr, axis):
        """Face fluxes of one direction from its face states (seam states
        already exchanged): x2 (axis 2) or x3 (axis 1)."""
        n, g = self.n, self.g
        fi = np.arange(NG, NG + n + 1)  # faces
        ri = np.arange(NG, NG + n)      # rows
        if axis == 2:
            cos, sin = g["cos_f2"][np.ix_(ri, fi)], g["sin_f2"][np.ix_(ri, fi)]
        else:
            cos, sin = g["cos_f3"][np.ix_(fi, ri)], g["sin_f3"][np.ix_(fi, ri)]
        wl, wr = wl.copy(), wr.copy()
        # to the face frame
        for w_ in (wl, wr):
            uu2, uu3 = w_[:, IVY].copy(), w_[:, IVZ].copy()
            if axis == 2:
                gi22 = 1.0 / (sin * sin)
                T22, T32, T33 = 1.0 / np.sqrt(gi22), cos / np.sqrt(1.0), np.sqrt(1.0)
                w_[:, IVZ] = T32 * uu2 + T33 * uu3
                w_[:, IVY] = T22 * uu2
            else:
                gi33 = 1.0 / (sin * sin)
                T22, T23, T33 = np.sqrt(1.0), cos / np.sqrt(1.0), 1.0 / np.sqrt(gi33)
                w_[:, IVY] = T22 * uu2 + T23 * uu3
                w_[:, IVZ] = T33 * uu3
        shape = wl.shape
        wl4 = np.moveaxis(wl, 1, -1)
        wr4 = np.moveaxis(wr, 1, -1)
        f = _roe(wl4, wr4, 2 if axis == 2 else 1, self.hllc).reshape(wl4.shape)
        f = np.moveaxis(f, -1, 1).copy()
        txy, txz = f[:, IVY].copy(), f[:, IVZ].copy()
        if axis == 2:
            gi22 = 1.0 / (sin * sin)
            T22 = np.sqrt(gi22)
            T32 = -np.sqrt(gi22) * cos / 1.0
            T33 = 1.0 / np.sqrt(1.0)
            f[:, IVZ] = T32 * txy + T33 * txz
            f[:, IVY] = T22 * txy
        else:
            gi33 = 1.0 / (sin * sin)
            T22 = 1.0 / np.sqrt(1.0)
            T23 = -cos / 1.0 * np.sqrt(gi33)
            T33 = np.sqrt(gi33)
            f[:, IVY] = T22 * txy + T23 * txz
            f[:, IVZ] = T33 * txz
        ty, tz = f[:, IVY].copy(), f[:, IVZ].copy()
        f[:, IVY] = ty + tz * cos
        f[:, IVZ] = tz + ty * cos
        assert f.shape == shape
        return f

    def fluxes(self, w):
        """Full face arrays F2 (6, 4, nc, nc+1), F3 (6, 4, nc+1, nc), zero
        outside the computed faces, seam faces single-valued."""
        n, nc = self.n, self.nc
        w2l, w2r = self._states(w, 2)
        w3l, w3r = self._states(w, 1)
        R.seam_states_all(w2l, w2r, w3l, w3r, self.g)
        F2 = np.zeros((6, 4, nc, nc + 1))
        F3 = np.zeros((6, 4, nc + 1, nc))
        F2[:, :, NG:NG + n, NG:NG + n + 1] = self._faces(w2l, w2r, 2)
        F3[:, :, NG:NG + n + 1, NG:NG + n] = self._faces(w3l, w3r, 1)
        R.reconcile(F2, F3, self.g)
        return F2, F3

    def tendency(self, u, dt):
        n, g = self.n, self.g
        w = self.cons2prim(u)
        F2, F3 = self.fluxes(w)
        self.last_fluxes = (F2, F3)
        I = slice(NG, NG + n)
        a2, a3 = g["area2"], g["area3"]
        d2 = a2[I, NG + 1:NG + n + 1] * F2[:, :, I, NG + 1:NG + n + 1] - \
            a2[I, NG:NG + n] * F2[:, :, I, NG:NG + n]
        d3 = a3[NG + 1:NG + n + 1, I] * F3[:, :, NG + 1:NG + n + 1, I] - \
            a3[NG:NG + n, I] * F3[:, :, NG:NG + n, I]
        div = (d2 + d3) / g["vol"][I, I]
        wi = w[:, :, I, I]
        pr = 0.5 * (wi[:, IDN] * wi[:, IDN])
        rho, v2, v3 = wi[:, IDN], wi[:, IVY], wi[:, IVZ]
        sine2 = g["sin_c"][I, I] * g["sin_c"][I, I]
        div[:, IVY] -= g["x_ov_rD"][I, I] * (pr + rho * v3 * v3 * sine2)
        div[:, IVZ] -= g["y_ov_rC"][I, I] * (pr + rho * v2 * v2 * sine2)
        du = np.zeros_like(u)
        du[:, :, I, I] = (-dt) * div
        return du

    def stage(self, u, u0, dt, s):
        if s == 0:
            u0[:] = u
        du = self.tendency(u, dt)
        w0, w1, w2 = self.wght[s]
        if self.steps is not None:
            n, I, J = self.n, slice(NG, NG + self.n), slice(NG, NG + self.n + 1)
            for d, F in zip((2, 3), self.last_fluxes):
                sel = (slice(None), slice(None), I, J) if d == 2 else \
                    (slice(None), slice(None), J, I)
                S = self.steps[d]
                S[sel] = (w2 * dt) * F[sel] if s == 0 else S[sel] * w1 + (w2 * dt) * F[sel]
        I = slice(NG, NG + self.n)
        u[:, :, I, I] = w0 * u0[:, :, I, I] + w1 * u[:, :, I, I] + w2 * du[:, :, I, I]
        self.fill(u)

    def max_dt(self, u):
        n, g = self.n, self.g
        I = slice(NG, NG + n)
        w = self.cons2prim(u)[:, :, I, I]
        cs = np.sqrt(w[:, IDN])
        d2 = g["width2"][I, I] / (np.abs(w[:, IVY]) + cs)
        d3 = g["width3"][I, I] / (np.abs(w[:, IVZ]) + cs)
        return self.cfl * min(d2.min(), d3.min())

    def mass(self, u):
        I = slice(NG, NG + self.n)
        return float((u[:, IDN, I, I] * self.g["vol"][I, I]).sum())
