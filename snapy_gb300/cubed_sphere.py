"""The cubed sphere: shallow water on six gnomonic-equiangle panels, one GPU.

Host side (numpy, FP64): the panel geometry and the two seam tables, built
once per grid and uploaded; device side (``csrc/sg_cs.cu``): the stage
(reconstruction, face-frame shallow-roe, seam flux single-valuing,
divergence with metric sources, RK combine) and the seam halo fill, driven
by those tables.

Geometry (src/coord/gnomonic_equiangle.cpp:38-259).  Every panel shares the
same angular grid: x2 = alpha, x3 = beta in [-pi/4, pi/4], N cells each way
(equal angles d = pi / 2N), nghost = 3, one radial cell [r, r + dr].  With
x = tan(alpha), y = tan(beta), C = sqrt(1 + x^2), D = sqrt(1 + y^2):
cos(theta) = -x y / (C D) (the angle between the alpha and beta lines),
sin(theta) = sqrt(1 + x^2 + y^2) / (C D); face lengths are arcs between the
face corners, a cell's x1 area its exact solid angle, and the metric source
factors x_ov_rD, y_ov_rC are the face-differences of (area sin) over the
volume.

Panels (src/layout/cubed_sphere_constants.h:43-80): the point of panel p at
(a, b) = (tan alpha, tan beta) is n_p + a e_a + b e_b, with
(n, e_a, e_b) = (+X, +Y, +Z), (+Y, -X, +Z), (-X, -Y, +Z), (+Z, +Y, -X),
(-Y, +X, +Z), (-Z, +Y, +X) for panels 0..5.

Seams (src/layout/cubed_sphere_layout.cpp:563-803, gnomonic_equiangle.cpp
:536-609).  A ghost centre beyond an edge lies on a grid line of the
neighbour panel at the matching depth; along the edge it falls between two
of the neighbour's cells.  The ghost takes the linear interpolation of those
two (written about the first, so equal values are returned exactly); its
momentum goes through the local geographic frame, as the reference's seam
exchange carries it (PanelRotation, src/coord/coord_rotation.cpp:105-147):
each source's covariant momentum is raised with its cell cosine to the unit
(alpha, beta) tangents and written in the (r, theta, phi) frame of its own
cell, those components are interpolated, and the ghost's covariant pair is
the vector with those components in the ghost's own frame, projected on the
ghost's tangents (covariant components are projections).  Seam face fluxes are made single-valued as
reconcile_panel_seams does (src/layout/seam_register.cpp:35): the lower
panel owns a seam, the other takes its flux, momentum rows rotated the same
way, with the sign flipped where both faces are the panels' low (or high)
sides.
"""
from __future__ import annotations

import math
from typing import Dict

import numpy as np

NG = 3
IDN, IVX, IVY, IVZ = 0, 1, 2, 3
SIDES = ("L", "R", "B", "T")  # alpha low / high, beta low / high

_X, _Y, _Z = np.eye(3)
FRAMES = [(_X, _Y, _Z), (_Y, -_X, _Z), (-_X, -_Y, _Z),
          (_Z, _Y, -_X), (-_Y, _X, _Z), (-_Z, _Y, _X)]

# doubles per ghost entry and per seam-face entry of the device tables
GHOST_STRIDE = 24
SEAM_STRIDE = 18


def geometry(n: int, r_in: float, dr: float = 1.0) -> Dict[str, np.ndarray]:
    """FP64 panel geometry on the padded grid, arrays indexed [k, j] (x3,
    x2); face arrays carry one more index along their direction."""
    import torch
    nc = n + 2 * NG
    d = 0.5 * math.pi / n
    # the faces as the reference lays a block's axis out: one linspace over
    # the global range widened by the ghosts (src/coord/coordinate.cpp:438)
    x2f = torch.linspace(-0.25 * math.pi - NG * d, 0.25 * math.pi + NG * d, nc + 1,
                         dtype=torch.float64).numpy()
    x2v = 0.5 * (x2f[:-1] + x2f[1:])
    x = np.tan(x2v)[None, :]
    xf = np.tan(x2f)[None, :]
    y = np.tan(x2v)[:, None]
    yf = np.tan(x2f)[:, None]
    C, Cf, D, Df = np.sqrt(1.0 + x * x), np.sqrt(1.0 + xf * xf), \
        np.sqrt(1.0 + y * y), np.sqrt(1.0 + yf * yf)
    g = {}
    g["cos_c"] = -x * y / (C * D)
    g["sin_c"] = np.sqrt(1.0 + x * x + y * y) / (C * D)
    g["cos_f2"] = -xf * y / (Cf * D)
    g["sin_f2"] = np.sqrt(1.0 + xf * xf + y * y) / (Cf * D)
    g["cos_f3"] = -x * yf / (C * Df)
    g["sin_f3"] = np.sqrt(1.0 + x * x + yf * yf) / (C * Df)

    def arc(e, a, b):
        e2 = e * e
        return np.arccos((1. + e2 + a * b) /
                         (np.sqrt(1. + e2 + a * a) * np.sqrt(1. + e2 + b * b)))

    x_lo, x_hi = np.tan(x2f[:-1])[None, :], np.tan(x2f[1:])[None, :]
    y_lo, y_hi = np.tan(x2f[:-1])[:, None], np.tan(x2f[1:])[:, None]
    dx2 = arc(y, x_lo, x_hi)        # [nc, nc]
    dx2_f3 = arc(yf, x_lo, x_hi)    # [nc + 1, nc]
    dx3 = arc(x, y_lo, y_hi)        # [nc, nc]
    dx3_f2 = arc(xf, y_lo, y_hi)    # [nc, nc + 1]
    corner = np.arctan(xf * yf / np.sqrt(1. + xf * xf + yf * yf))
    solid = corner[1:, 1:] - corner[1:, :-1] - corner[:-1, 1:] + corner[:-1, :-1]
    rm, rp = r_in, r_in + dr
    x1v = 0.5 * (rm + rp)
    rad = x1v * dr
    g["area2"] = rad * dx3_f2
    g["area3"] = rad * dx2_f3
    g["vol"] = (dr * (rp * rp + rp * rm + rm * rm) / 3.0) * solid
    fx = g["area2"] * g["sin_f2"]
    fy = g["area3"] * g["sin_f3"]
    g["x_ov_rD"] = (fx[:, 1:] - fx[:, :-1]) / g["vol"]
    g["y_ov_rC"] = (fy[1:, :] - fy[:-1, :]) / g["vol"]
    g["width2"] = x1v * dx2
    g["width3"] = x1v * dx3
    g["x2v"], g["x2f"], g["radius"] = x2v, x2f, x1v
    return {k: np.ascontiguousarray(v) if isinstance(v, np.ndarray) else v
            for k, v in g.items()}


def point(p: int, alpha, beta) -> np.ndarray:
    """Unit position vectors [..., 3] of panel p at (alpha, beta)."""
    n, ea, eb = FRAMES[p]
    a, b = np.tan(alpha), np.tan(beta)
    P = n + np.asarray(a)[..., None] * ea + np.asarray(b)[..., None] * eb
    return P / np.linalg.norm(P, axis=-1, keepdims=True)


def tangents(p: int, alpha, beta):
    """The unit tangents of the alpha and beta lines of panel p [..., 3]."""
    n, ea, eb = FRAMES[p]
    a, b = np.asarray(np.tan(alpha)), np.asarray(np.tan(beta))
    P = n + a[..., None] * ea + b[..., None] * eb
    P2 = np.sum(P * P, axis=-1, keepdims=True)
    ta = ea - P * (np.sum(P * ea, axis=-1, keepdims=True) / P2)
    tb = eb - P * (np.sum(P * eb, axis=-1, keepdims=True) / P2)
    ta /= np.linalg.norm(ta, axis=-1, keepdims=True)
    tb /= np.linalg.norm(tb, axis=-1, keepdims=True)
    return ta, tb


def geo_frame(P: np.ndarray):
    """The local geographic frame (r, theta, phi) at unit positions P
    [..., 3]: r = P, theta = (x z / s, y z / s, -s), phi = (-y / s, x / s,
    0), s = sqrt(x^2 + y^2) (the frame of PanelRotation,
    src/coord/coord_rotation.cpp:12-58; no cell centre or ghost of an
    even-sized grid lies on a pole)."""
    x, y, z = P[..., 0], P[..., 1], P[..., 2]
    s = np.sqrt(x * x + y * y)
    th = np.stack([x * z / s, y * z / s, -s], axis=-1)
    ph = np.stack([-y / s, x / s, np.zeros_like(s)], axis=-1)
    return P, th, ph


def on_panel(q: int, P: np.ndarray):
    """(alpha, beta) of unit vectors P on panel q (P . n_q > 0)."""
    n, ea, eb = FRAMES[q]
    pn = P @ n
    return np.arctan((P @ ea) / pn), np.arctan((P @ eb) / pn)


def _neighbour(p: int, P: np.ndarray) -> int:
    dots = [float(np.mean(P @ FRAMES[q][0])) if q != p else -2. for q in range(6)]
    return int(np.argmax(dots))


def _side_cells(side: str, n: int, depth: int, along: np.ndarray):
    """Padded (k, j) of ghost cells of a side at a depth, and their angles."""
    d = 0.5 * math.pi / n
    perp = 0.25 * math.pi + (depth - 0.5) * d
    cen = -0.25 * math.pi + (along + 0.5) * d
    if side == "L":
        return NG + along, np.full_like(along, NG - depth), np.full(along.shape, -perp), cen
    if side == "R":
        return NG + along, np.full_like(along, NG + n - 1 + depth), np.full(along.shape, perp), cen
    if side == "B":
        return np.full_like(along, NG - depth), NG + along, cen, np.full(along.shape, -perp)
    return np.full_like(along, NG + n - 1 + depth), NG + along, cen, np.full(along.shape, perp)


def ghost_table(n: int, geo: Dict[str, np.ndarray]) -> np.ndarray:
    """One row of GHOST_STRIDE doubles per seam ghost cell:
    [dst flat index, src0 flat index, src1 flat index, x (the fraction toward
    src1), cos0, ta0[3], tb0[3], cos1, ta1[3], tb1[3], ta_g[3], tb_g[3]].
    Flat index = (panel * nc + k) * nc + j of a cell of the padded panel."""
    nc = n + 2 * NG
    d = 0.5 * math.pi / n
    rows = []
    along = np.arange(n)
    for p in range(6):
        for side in SIDES:
            for depth in range(1, NG + 1):
                kd, jd, al, be = _side_cells(side, n, depth, along)
                P = point(p, al, be)
                q = _neighbour(p, P)
                aq, bq = on_panel(q, P)
                ia = (aq + 0.25 * math.pi) / d - 0.5
                ib = (bq + 0.25 * math.pi) / d - 0.5
                # the perpendicular index is the same for the whole edge
                if np.ptp(ia) < 1e-6:
                    perp, u, perp_is_a = ia, ib, True
                else:
                    perp, u, perp_is_a = ib, ia, False
                pi_ = int(round(float(perp[0])))
                assert np.max(np.abs(perp - pi_)) < 1e-6, (p, side, depth)
                u0 = np.clip(np.floor(u), 0, n - 2).astype(int)
                x = u - u0
                # the ghost's covariant pair from geographic components:
                # m2 = V . ta_g with V = V_r r + V_th th + V_ph ph (at the
                # ghost), so its row is (ta_g . r, ta_g . th, ta_g . ph)
                ta_g, tb_g = tangents(p, al, be)
                fr_g = geo_frame(P)
                rows_a = np.stack([np.sum(ta_g * e, -1) for e in fr_g], -1)
                rows_b = np.stack([np.sum(tb_g * e, -1) for e in fr_g], -1)
                for m in range(n):
                    srcs = []
                    for s in (u0[m], u0[m] + 1):
                        jj, kk = (pi_, s) if perp_is_a else (s, pi_)
                        srcs.append((q, NG + kk, NG + jj))
                    row = [(p * nc + kd[m]) * nc + jd[m]]
                    row += [(sq * nc + sk) * nc + sj for sq, sk, sj in srcs]
                    row += [x[m]]
                    for sq, sk, sj in srcs:
                        # a source's contravariant pair to geographic
                        # components at the source cell: the unit tangents
                        # written in its (r, theta, phi) frame
                        a_s, b_s = geo["x2v"][sj], geo["x2v"][sk]
                        ta, tb = tangents(sq, a_s, b_s)
                        fr = geo_frame(point(sq, a_s, b_s))
                        row += [geo["cos_c"][sk, sj]]
                        row += [float(np.dot(ta, e)) for e in fr]
                        row += [float(np.dot(tb, e)) for e in fr]
                    row += list(rows_a[m]) + list(rows_b[m])
                    rows.append(row)
    t = np.array(rows, dtype=np.float64)
    assert t.shape[1] == GHOST_STRIDE
    return np.ascontiguousarray(t)


def seam_table(n: int, geo: Dict[str, np.ndarray]) -> np.ndarray:
    """One row of SEAM_STRIDE doubles per seam face that takes its flux
    from the owning (lower) panel:
    [dst dir (2 or 3), dst flat face index, src dir, src flat face index,
    sign, cos_src, ta_src[3], tb_src[3], ta_dst[3], tb_dst[3]].
    Face flat index = (panel * nk + k) * nj + j of that direction's face
    array (x2 faces: nk = nc, nj = nc + 1; x3 faces: nk = nc + 1, nj = nc)."""
    nc = n + 2 * NG
    d = 0.5 * math.pi / n
    cen = -0.25 * math.pi + (np.arange(n) + 0.5) * d
    edge = 0.25 * math.pi

    def faces(p, side):
        """(dir, k, j, alpha, beta) of the n faces of a side of panel p."""
        m = np.arange(n)
        if side == "L":
            return 2, NG + m, np.full(n, NG), np.full(n, -edge), cen
        if side == "R":
            return 2, NG + m, np.full(n, NG + n), np.full(n, edge), cen
        if side == "B":
            return 3, np.full(n, NG), NG + m, cen, np.full(n, -edge)
        return 3, np.full(n, NG + n), NG + m, cen, np.full(n, edge)

    def flat(dirn, p, k, j):
        return (p * nc + k) * (nc + 1) + j if dirn == 2 else (p * (nc + 1) + k) * nc + j

    rows = []
    for p in range(6):
        for side in SIDES:
            dirn, k, j, al, be = faces(p, side)
            P = point(p, al, be)
            q = _neighbour(p, point(p, al * 1.01, be * 1.01))
            if q > p:
                continue  # p owns this seam
            aq, bq = on_panel(q, P)
            # the matching side of q and the along index of each face
            if np.ptp(aq) < 1e-9 and abs(abs(aq[0]) - edge) < 1e-9:
                qside = "L" if aq[0] < 0 else "R"
                m_q = np.rint((bq + edge) / d - 0.5).astype(int)
            else:
                assert np.ptp(bq) < 1e-9 and abs(abs(bq[0]) - edge) < 1e-9
                qside = "B" if bq[0] < 0 else "T"
                m_q = np.rint((aq + edge) / d - 0.5).astype(int)
            qdir, qk, qj, qal, qbe = faces(q, qside)
            sign = -1.0 if (SIDES.index(side) % 2) == (SIDES.index(qside) % 2) else 1.0
            ta_d, tb_d = tangents(p, al, be)
            for m in range(n):
                mq = m_q[m]
                ta_s, tb_s = tangents(q, qal[mq], qbe[mq])
                cs = (geo["cos_f2"][qk[mq], qj[mq]] if qdir == 2
                      else geo["cos_f3"][qk[mq], qj[mq]])
                rows.append([dirn, flat(dirn, p, k[m], j[m]), qdir,
                             flat(qdir, q, qk[mq], qj[mq]), sign, cs]
                            + list(ta_s) + list(tb_s) + list(ta_d[m]) + list(tb_d[m]))
    t = np.array(rows, dtype=np.float64)
    assert t.shape[1] == SEAM_STRIDE
    return np.ascontiguousarray(t)


SEAM_STATE_STRIDE = 16


def _side_faces(p: int, side: str, n: int):
    """(alpha, beta) of the n interior faces of a side of panel p."""
    d = 0.5 * math.pi / n
    cen = -0.25 * math.pi + (np.arange(n) + 0.5) * d
    e = 0.25 * math.pi
    if side in ("L", "R"):
        return np.full(n, -e if side == "L" else e), cen
    return cen, np.full(n, -e if side == "B" else e)


def seam_state_table(n: int) -> np.ndarray:
    """One row of SEAM_STATE_STRIDE doubles per seam face, ordered (panel,
    side L R B T, along): the neighbour panel q sharing the face, q's side
    (0..3 for L R B T) and the face's along index on it (so the seam buffer
    row (4 q + side) n + along holds q's own interior-side state there), a
    0, and the 3 x 3 map (row major) of contravariant velocities (radial,
    alpha, beta) in q's unit basis at the face to this panel's:
    M = B_p^-1 B_q with B the basis (r, t_alpha, t_beta) as columns."""
    d = 0.5 * math.pi / n
    e = 0.25 * math.pi
    rows = np.zeros((6, 4, n, SEAM_STATE_STRIDE))
    for p in range(6):
        for si, side in enumerate(SIDES):
            al, be = _side_faces(p, side, n)
            P = point(p, al, be)
            # the neighbour: the panel just beyond the edge
            out = 1.01
            q = _neighbour(p, point(p, al * out if side in "LR" else al,
                                    be * out if side in "BT" else be))
            aq, bq = on_panel(q, P)
            if np.ptp(aq) < 1e-9 and abs(abs(aq[0]) - e) < 1e-9:
                qside = "L" if aq[0] < 0 else "R"
                mq = np.rint((bq + e) / d - 0.5).astype(int)
            else:
                assert np.ptp(bq) < 1e-9 and abs(abs(bq[0]) - e) < 1e-9
                qside = "B" if bq[0] < 0 else "T"
                mq = np.rint((aq + e) / d - 0.5).astype(int)
            ta_p, tb_p = tangents(p, al, be)
            ta_q, tb_q = tangents(q, aq, bq)
            for m in range(n):
                Bp = np.stack([P[m], ta_p[m], tb_p[m]], axis=1)
                Bq = np.stack([P[m], ta_q[m], tb_q[m]], axis=1)
                M = np.linalg.solve(Bp, Bq)
                rows[p, si, m, :4] = (q, SIDES.index(qside), mq[m], 0)
                rows[p, si, m, 4:13] = M.ravel()
    return np.ascontiguousarray(rows.reshape(-1, SEAM_STATE_STRIDE))


def lonlat(p: int, alpha, beta):
    """Longitude and latitude of panel p's points."""
    P = point(p, alpha, beta)
    return np.arctan2(P[..., 1], P[..., 0]), np.arcsin(np.clip(P[..., 2], -1., 1.))


def bump(n: int, radius: float = 6.371e6, seed: int = 0, depth: float = 1000.,
         height: float = 100., width: float = 0.1, grav: float = 9.81) -> np.ndarray:
    """The cubed-sphere initial state (6, 4, nc, nc) FP64, conserved: mean
    geopotential grav depth, a Gaussian bump grav height exp(-d^2 / width^2)
    in the great-circle distance d (radians) from a centre drawn, from a
    generator seeded with `seed`, uniformly in lon [-pi, pi), lat [-pi/3,
    pi/3]; at rest.  Ghosts are left zero (the seam fill sets them)."""
    import torch
    gen = torch.Generator().manual_seed(int(seed))
    lon0 = float((torch.rand(1, generator=gen, dtype=torch.float64) * 2. - 1.) * math.pi)
    lat0 = float((torch.rand(1, generator=gen, dtype=torch.float64) * 2. - 1.) * math.pi / 3.)
    nc = n + 2 * NG
    d = 0.5 * math.pi / n
    c = -0.25 * math.pi + (np.arange(n) + 0.5) * d
    beta, alpha = np.meshgrid(c, c, indexing="ij")
    u = np.zeros((6, 4, nc, nc))
    for p in range(6):
        lon, lat = lonlat(p, alpha, beta)
        cosd = np.sin(lat) * math.sin(lat0) + np.cos(lat) * math.cos(lat0) * np.cos(lon - lon0)
        dist = np.arccos(np.clip(cosd, -1., 1.))
        u[p, IDN, NG:NG + n, NG:NG + n] = grav * depth + grav * height * np.exp(-(dist / width) ** 2)
    return u


RK3 = ((1.0, 0.0, 1.0), (0.75, 0.25, 0.25), (1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0))

# the order of the geometry arrays in the device block (sg_cs_desc.geo)
GEO_ORDER = ("cos_c", "sin_c", "vol", "x_ov_rD", "y_ov_rC", "width2", "width3",
             "cos_f2", "sin_f2", "area2", "cos_f3", "sin_f3", "area3")


class SphereSW:
    """Shallow water on the six panels, one handle on one GPU.

    state (6, 4, n + 6, n + 6) in the dtype: Phi, the radial and the two
    covariant tangential momenta; the RK stages rotate three such buffers.
    In FP32 the stored Phi row is the anomaly Phi - phi_ref (the geopotential
    of the mean depth) and the pressure is carried as an anomaly about it:
    ``totals()`` gives the FP64 totals.
    ``step`` advances one RK3 step with the device CFL time step (a captured
    graph after the first steps of each buffer rotation)."""

    def __init__(self, n: int, radius: float = 6.371e6, dtype=None, device=None,
                 wght=RK3, cfl: float = 0.9, graphs: bool = True,
                 phi_ref: float = 9.81 * 1000.0, riemann: str = "shallow-roe"):
        import ctypes
        import torch
        from . import _lib
        self.torch = torch
        self.L = _lib.load()
        self.n, self.nc = n, n + 2 * NG
        self.dtype = dtype or torch.float32
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        self.geo = geometry(n, radius)
        gt = ghost_table(n, self.geo)
        st = seam_table(n, self.geo)
        sst = seam_state_table(n)
        dev = self.device
        self._geo = torch.as_tensor(np.concatenate([self.geo[k].ravel() for k in GEO_ORDER]),
                                    dtype=torch.float64, device=dev)
        self._gt = torch.as_tensor(gt, dtype=torch.float64, device=dev)
        self._st = torch.as_tensor(st, dtype=torch.float64, device=dev)
        self._sst = torch.as_tensor(sst, dtype=torch.float64, device=dev)
        d = _lib.CsDesc()
        d.n, d.ng = n, NG
        d.dtype = _lib.F64 if self.dtype == torch.float64 else _lib.F32
        d.nstage = len(wght)
        for s_, w in enumerate(wght):
            for q in range(3):
                d.wght[s_][q] = w[q]
        d.cfl = cfl
        d.geo, d.ghost_tab, d.seam_tab = (self._geo.data_ptr(), self._gt.data_ptr(),
                                          self._st.data_ptr())
        d.nghost, d.nseam = gt.shape[0], st.shape[0]
        d.seam_state_tab, d.nseam_state = self._sst.data_ptr(), sst.shape[0]
        # FP32: the pressure as an anomaly about Phi0 (the mean depth's
        # geopotential); FP64 keeps the reference's form
        d.phi_ref = float(phi_ref)
        if riemann not in ("shallow-roe", "hllc"):
            raise ValueError(f"riemann-solver '{riemann}': shallow-roe or hllc")
        d.riemann = 1 if riemann == "hllc" else 0
        self.nstage = len(wght)
        h = ctypes.c_void_p()
        with torch.cuda.device(dev):
            _lib.check(self.L.sg_cs_create(ctypes.byref(d), ctypes.byref(h)), "sg_cs_create")
        self.h = h
        self.store = torch.zeros((3, 6, 4, self.nc, self.nc), dtype=self.dtype, device=dev)
        nb = ctypes.c_size_t()
        _lib.check(self.L.sg_cs_scratch_bytes(h, ctypes.byref(nb)), "sg_cs_scratch_bytes")
        self.scratch = torch.empty((nb.value + 7) // 8, dtype=torch.float64, device=dev)
        _lib.check(self.L.sg_cs_bind(h, *(self.store[q].data_ptr() for q in range(3)),
                                     self.scratch.data_ptr(), self.scratch.numel() * 8),
                   "sg_cs_bind")
        _lib.check(self.L.sg_cs_set_current(h, 0), "sg_cs_set_current")
        self.dt = torch.zeros(1, dtype=torch.float64, device=dev)
        self.phi0 = float(phi_ref) if self.dtype == torch.float32 else 0.0
        self.graphs = graphs
        self._graphs, self._seen = {}, set()
        self.replays = self.captures = 0
        self.time = 0.0

    def close(self):
        if getattr(self, "h", None):
            self.L.sg_cs_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _stream(self):
        return self.torch.cuda.current_stream(self.device).cuda_stream

    def rotation(self):
        import ctypes
        c, b = ctypes.c_int32(), ctypes.c_int32()
        self._chk(self.L.sg_cs_rotation(self.h, ctypes.byref(c), ctypes.byref(b)), "sg_cs_rotation")
        return c.value, b.value

    def _chk(self, rc, what):
        from . import _lib
        _lib.check(rc, what)

    def request_step_field(self, dim: int):
        """The FluxRegister's step fields (both directions are kept):
        S_d <- w1 S_d + w2 dt T_d over the stage's final face fluxes, FP64,
        (6, 4, nc, nc + 1) for d = 2 and (6, 4, nc + 1, nc) for d = 3, face
        j of row k at [..., k, j]; zero at stage 0 of every step."""
        if dim not in (2, 3):
            raise ValueError("the cubed sphere's step fields are d = 2, 3")
        torch = self.torch
        if getattr(self, "_steps", None) is None:
            nc = self.nc
            self._steps = {
                2: torch.zeros((6, 4, nc, nc + 1), dtype=torch.float64, device=self.device),
                3: torch.zeros((6, 4, nc + 1, nc), dtype=torch.float64, device=self.device)}
            self._chk(self.L.sg_cs_bind_step_fields(self.h, self._steps[2].data_ptr(),
                                                    self._steps[3].data_ptr()),
                      "sg_cs_bind_step_fields")
            self._graphs.clear()  # captured before the fields existed
        return self._steps[dim]

    def step_field(self, dim: int):
        return self._steps[dim]

    def budget_totals(self):
        """The row totals sum u V over the interior cells (Phi, the radial
        and the two tangential momenta), FP64, on the device."""
        torch = self.torch
        out = torch.empty(4, dtype=torch.float64, device=self.device)
        with torch.cuda.device(self.device):
            self._chk(self.L.sg_cs_budget_totals(self.h, out.data_ptr(), self._stream()),
                      "sg_cs_budget_totals")
        return out

    def state(self):
        """The current conserved state (a view of the handle's buffer)."""
        return self.store[self.rotation()[0]]

    def initialize(self, u) -> None:
        """Load a conserved state (6, 4, nc, nc) (its interior; the seam halo
        is filled here)."""
        with self.torch.cuda.device(self.device):
            self._chk(self.L.sg_cs_set_current(self.h, 0), "sg_cs_set_current")
            u = self.torch.as_tensor(u).to(self.device, self.torch.float64).clone()
            if self.phi0:
                u[:, IDN] -= self.phi0  # the stored anomaly, formed in FP64
            self.store[0].copy_(u.to(self.dtype))
            self._chk(self.L.sg_cs_fill_seams(self.h, self._stream()), "sg_cs_fill_seams")
        self.time = 0.0

    def max_dt(self):
        with self.torch.cuda.device(self.device):
            self._chk(self.L.sg_cs_max_dt(self.h, self.dt.data_ptr(), self._stream()),
                      "sg_cs_max_dt")
        return self.dt

    def _launch(self, fixed):
        if fixed is None:
            self.L.sg_cs_max_dt(self.h, self.dt.data_ptr(), self._stream())
        else:
            self.dt.copy_(fixed)
        for s_ in range(self.nstage):
            self._chk(self.L.sg_cs_stage(self.h, s_, self.dt.data_ptr(), self._stream()),
                      "sg_cs_stage")

    def step(self, dt: "float | None" = None) -> None:
        """One RK step: the device CFL dt (or the given dt), all stages."""
        torch = self.torch
        with torch.cuda.device(self.device):
            fixed = None if dt is None else torch.full((1,), float(dt), dtype=torch.float64,
                                                      device=self.device)
            rot = self.rotation()
            key = (rot, dt is None)
            g = self._graphs.get(key) if self.graphs else None
            if g is None and self.graphs and key in self._seen:
                g = torch.cuda.CUDAGraph()
                buf = torch.zeros(1, dtype=torch.float64, device=self.device)
                s = torch.cuda.Stream(device=self.device)
                s.wait_stream(torch.cuda.current_stream())
                try:
                    with torch.cuda.stream(s):
                        g.capture_begin()
                        try:
                            self._launch(None if dt is None else buf)
                        finally:
                            g.capture_end()
                finally:
                    self._chk(self.L.sg_cs_set_rotation(self.h, *rot), "sg_cs_set_rotation")
                torch.cuda.current_stream().wait_stream(s)
                g = (g, buf)
                self._graphs[key] = g
                self.captures += 1
            if g is not None:
                graph, buf = g
                if fixed is not None:
                    buf.copy_(fixed)
                graph.replay()
                for s_ in range(self.nstage):
                    self._chk(self.L.sg_cs_advance(self.h, s_), "sg_cs_advance")
                self.replays += 1
            else:
                self._launch(fixed)
                self._seen.add(key)

    def totals(self):
        """The current conserved state with Phi as a total (FP64)."""
        u = self.state().double()
        if self.phi0:
            u[:, IDN] += self.phi0
        return u

    def mass(self) -> float:
        """The total of Phi over the six panels' interiors, times the cell
        volume (FP64 on the host)."""
        u = self.totals()[:, IDN, NG:NG + self.n, NG:NG + self.n].cpu().numpy()
        return float((u * self.geo["vol"][NG:NG + self.n, NG:NG + self.n]).sum())
