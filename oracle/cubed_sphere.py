"""CPU restatement of the cubed-sphere shallow-water stage (FP64): TEST
INFRASTRUCTURE ONLY -- the checker of the GPU path, never part of it.

The array plumbing is numpy; the pointwise reconstruction (WENO5 / cp5) and
the shallow-roe solver are the C oracle's (oracle/sg_oracle.c), pinned to the
reference's kernels.  The grid geometry and the two seam tables are inputs,
built by snapy_gb300.cubed_sphere on the host, as the Cartesian oracle takes
its x1 faces; the tables are checked separately against analytic fields.

One stage follows the reference (src/hydro/hydro_forward.cpp with the
gnomonic coordinate of src/coord/gnomonic_equiangle.cpp):
  W = U/Phi with the momenta raised by the cell cosine (ShallowWaterImpl::
  _cons2prim, src/eos/shallow_water.cpp:30-42; coord_vec_raise_impl,
  src/coord/coord_utils_impl.h:9-16);
  x2 / x3 face states, weno5 for Phi and cp5 for the velocities
  (reconstruct.cpp:151-187);
  to the face frame (prim2local2_/3_, gnomonic_equiangle.cpp:357-398),
  shallow_roe with dir yz (riemann_kernels.h:447-495) or the product's
  shallow-water HLLC (og_hllc_sw_batch), back to covariant
  fluxes (flux2global2_/3_, :414-463);
  the seam faces single-valued (src/layout/seam_register.cpp:35);
  div = (A2 dF2 + A3 dF3) / V (coordinate.cpp:618-662), minus the metric
  sources x_ov_rD (p + Phi v3 v3 sin^2), y_ov_rC (p + Phi v2 v2 sin^2),
  p = Phi^2 / 2 (gnomonic_equiangle.cpp:465-521); du = -dt div;
  the RK combine, then the seam halo fill.
"""
from __future__ import annotations

import numpy as np

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
    covariant tangential momenta."""

    def __init__(self, n, geo, ghost_tab, seam_tab, wght, cfl, riemann="shallow-roe"):
        self.n, self.g = n, geo
        self.hllc = riemann == "hllc"
        self.gt, self.st = ghost_tab, seam_tab
        self.wght, self.cfl = wght, cfl
        self.nc = n + 2 * NG

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
        t = self.gt
        flat = u.transpose(1, 0, 2, 3).reshape(4, -1)
        d, s0, s1 = t[:, 0].astype(np.int64), t[:, 1].astype(np.int64), t[:, 2].astype(np.int64)
        x = t[:, 3]
        for v in (IDN, IVX):
            a, b = flat[v, s0], flat[v, s1]
            flat[v, d] = a + x * (b - a)

        def glob(idx, c, ta, tb):
            m2, m3 = flat[IVY, idx], flat[IVZ, idx]
            s2 = 1. - c * c
            v2 = m2 / s2 - m3 * c / s2
            v3 = -m2 * c / s2 + m3 / s2
            return [ta[:, q] * v2 + tb[:, q] * v3 for q in range(3)]

        V0 = glob(s0, t[:, 4], t[:, 5:8], t[:, 8:11])
        V1 = glob(s1, t[:, 11], t[:, 12:15], t[:, 15:18])
        V = [V0[q] + x * (V1[q] - V0[q]) for q in range(3)]
        ta, tb = t[:, 18:21], t[:, 21:24]
        flat[IVY, d] = (V[0] * ta[:, 0] + V[1] * ta[:, 1]) + V[2] * ta[:, 2]
        flat[IVZ, d] = (V[0] * tb[:, 0] + V[1] * tb[:, 1]) + V[2] * tb[:, 2]
        u[:] = flat.reshape(4, 6, self.nc, self.nc).transpose(1, 0, 2, 3)

    def _faces(self, w, axis):
        """Face fluxes of one direction: x2 (axis 2: faces j = NG..NG+n of
        rows k = NG..NG+n-1) or x3 (axis 1)."""
        n, g = self.n, self.g
        fi = np.arange(NG, NG + n + 1)  # faces
        ri = np.arange(NG, NG + n)      # rows
        if axis == 2:
            st = np.stack([w[:, :, ri][:, :, :, fi + o] for o in range(-3, 3)], -1)
            cos, sin = g["cos_f2"][np.ix_(ri, fi)], g["sin_f2"][np.ix_(ri, fi)]
        else:
            st = np.stack([w[:, :, fi + o][:, :, :, ri] for o in range(-3, 3)], -1)
            cos, sin = g["cos_f3"][np.ix_(fi, ri)], g["sin_f3"][np.ix_(fi, ri)]
        # st: (6, 4, rows/faces..., 6 cells)
        wl = np.empty(st.shape[:-1])
        wr = np.empty(st.shape[:-1])
        for v in range(4):
            weno = v == IDN
            wl[:, v] = _recon(st[:, v, ..., 0:5], weno, 1).reshape(wl[:, v].shape)
            wr[:, v] = _recon(st[:, v, ..., 1:6], weno, 0).reshape(wr[:, v].shape)
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
        F2 = np.zeros((6, 4, nc, nc + 1))
        F3 = np.zeros((6, 4, nc + 1, nc))
        F2[:, :, NG:NG + n, NG:NG + n + 1] = self._faces(w, 2)
        F3[:, :, NG:NG + n + 1, NG:NG + n] = self._faces(w, 1)
        f2 = F2.transpose(1, 0, 2, 3).reshape(4, -1)
        f3 = F3.transpose(1, 0, 2, 3).reshape(4, -1)
        src = {2: f2.copy(), 3: f3.copy()}
        for row in self.st:
            dd, di, sd, si, sign, c = int(row[0]), int(row[1]), int(row[2]), int(row[3]), row[4], row[5]
            ta_s, tb_s, ta_d, tb_d = row[6:9], row[9:12], row[12:15], row[15:18]
            s = src[sd]
            dst = f2 if dd == 2 else f3
            m2, m3 = s[IVY, si], s[IVZ, si]
            s2 = 1. - c * c
            v2 = m2 / s2 - m3 * c / s2
            v3 = -m2 * c / s2 + m3 / s2
            V = [ta_s[q] * v2 + tb_s[q] * v3 for q in range(3)]
            dst[IDN, di] = sign * s[IDN, si]
            dst[IVX, di] = sign * s[IVX, si]
            dst[IVY, di] = sign * ((V[0] * ta_d[0] + V[1] * ta_d[1]) + V[2] * ta_d[2])
            dst[IVZ, di] = sign * ((V[0] * tb_d[0] + V[1] * tb_d[1]) + V[2] * tb_d[2])
        F2 = f2.reshape(4, 6, nc, nc + 1).transpose(1, 0, 2, 3)
        F3 = f3.reshape(4, 6, nc + 1, nc).transpose(1, 0, 2, 3)
        return F2, F3

    def tendency(self, u, dt):
        n, g = self.n, self.g
        w = self.cons2prim(u)
        F2, F3 = self.fluxes(w)
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
