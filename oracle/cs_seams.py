"""The reference's cubed-sphere geometry and panel-seam exchanges, restated
in numpy (FP64): TEST INFRASTRUCTURE ONLY -- the checker of the GPU path.

Nothing here comes from the product's own tables: every quantity is built
from the reference's definitions, one function per reference routine.

* geometry(): GnomonicEquiangleImpl::reset (src/coord/gnomonic_equiangle.cpp
  :38-259) -- faces from the global linspace (src/coord/coordinate.cpp
  :425-445), the cell and face metric cosines and sines, arc face lengths,
  exact solid angles and volumes (:298-308), the metric source factors.
* contra_to_cart / cart_to_contra: cs_contra_to_cart_at_ /
  cs_cart_to_contra_at_ (src/coord/cubed_sphere_utils.cpp:213-256) with the
  CS_LOCAL_TO_CART_VEL / CS_CART_TO_LOCAL_VEL tables
  (src/layout/cubed_sphere_constants.h:23-40); raise / lower:
  coord_vec_raise_impl / coord_vec_lower_impl (src/coord/coord_utils_impl.h).
* rotation(): PanelRotation::matrix (src/coord/coord_rotation.cpp:105-147):
  a panel's components to the local geographic frame (r, theta, phi) of the
  point and back (local_frame, cart_to_local_, local_to_cart_ :12-58).
* usrc(): cs_build_ghost_usrc (src/coord/cubed_sphere_utils.cpp:78-108) with
  cs_equ_ghost_center, cs_xyz_to_ab and cs_angle_to_center_u; the reference
  builds it once, for face 0's left side, and every block uses that table.
* fill(): the cross-panel ghost exchange of hydro_u (kConserved) with one
  block per panel: CubedSphereLayoutImpl::serialize (the neighbour's
  interior strip widened by the interpolation margin, its momenta to the
  geographic frame at its own cells, then the rev / flip / transpose of its
  buffer, src/layout/cubed_sphere_layout.cpp:563-700), deserialize (the raw
  copy into the wide landing zone, interp_ghost, the momenta back to the
  receiver's covariant components at its ghost cells, :702-803) and
  _interp_ghost (linear along the edge about the first source,
  src/coord/gnomonic_equiangle.cpp:536-609).
* seam_states(): the face-state exchange of the x2 / x3 sweeps
  (src/hydro/hydro_forward.cpp:719-757): at a panel seam each panel's
  exterior-side state is the neighbour panel's own interior-side state at
  the same face (kPrimitive: contravariant velocities, no cosine).
* reconcile(): reconcile_panel_seams (src/layout/seam_register.cpp:35-177):
  the lower panel owns a seam face; the other takes its face fluxes through
  the Cartesian frame, reversed along the edge where the connectivity says
  so and negated where both sides are low (or both high) sides.
"""
from __future__ import annotations

import math

import numpy as np

NG = 3
IDN, IVX, IVY, IVZ = 0, 1, 2, 3
SIDE_L, SIDE_R, SIDE_B, SIDE_T = 0, 1, 2, 3

# leaving face F by side S arrives at (face, side, along-edge reversed)
# (src/layout/cubed_sphere_layout.cpp CS_FACE_EDGES)
FACE_EDGES = (
    ((4, SIDE_R, 0), (1, SIDE_L, 0), (5, SIDE_T, 0), (3, SIDE_B, 0)),
    ((0, SIDE_R, 0), (2, SIDE_L, 0), (5, SIDE_R, 1), (3, SIDE_R, 0)),
    ((1, SIDE_R, 0), (4, SIDE_L, 0), (5, SIDE_B, 1), (3, SIDE_T, 1)),
    ((4, SIDE_T, 1), (1, SIDE_T, 0), (0, SIDE_T, 0), (2, SIDE_T, 1)),
    ((2, SIDE_R, 0), (0, SIDE_L, 0), (5, SIDE_L, 0), (3, SIDE_L, 1)),
    ((4, SIDE_B, 0), (1, SIDE_B, 1), (2, SIDE_B, 1), (0, SIDE_B, 0)),
)

# Cartesian components are stored (z, x, y) in slots 0..2 (VEL1..VEL3).
# cart -> panel-local Cartesian: local[idx[f][c]] = sgn[f][c] * cart[c]
C2L_IDX = ((2, 0, 1), (2, 1, 0), (2, 0, 1), (0, 2, 1), (2, 1, 0), (0, 2, 1))
C2L_SGN = ((1, 1, 1), (1, -1, 1), (1, -1, -1), (1, -1, 1), (1, 1, -1), (-1, 1, 1))
# panel-local -> cart: cart[idx[f][c]] = sgn[f][c] * (local expression c)
L2C_IDX = ((1, 2, 0), (2, 1, 0), (1, 2, 0), (0, 2, 1), (2, 1, 0), (0, 2, 1))
L2C_SGN = ((1, 1, 1), (1, -1, 1), (-1, -1, 1), (1, 1, -1), (-1, 1, 1), (-1, 1, 1))


def face_xyz(face, a, b):
    """cs_face_xyz_from_tan (src/layout/cubed_sphere_constants.h:43-80)."""
    one = np.ones_like(a)
    return {0: (one, a, b), 1: (-a, one, b), 2: (-one, -a, b),
            3: (-b, a, one), 4: (a, -one, b), 5: (b, a, -one)}[face]


def _metric(alpha, beta):
    x, y = np.tan(alpha), np.tan(beta)
    return x, y, np.sqrt(x * x + y * y + 1), np.sqrt(1 + x * x), np.sqrt(1 + y * y)


def contra_to_cart(v, face, alpha, beta):
    """v: [3, ...] contravariant (unit alpha / beta basis, radial first) ->
    Cartesian (z, x, y)."""
    x, y, delta, C, D = _metric(alpha, beta)
    vz, vx, vy = v[0], v[1], v[2]
    loc = ((vz - vx * x / D - vy * y / C) / delta,
           (vz * x + vx * D - (vy * x * y) / C) / delta,
           (vz * y + vy * C - (vx * x * y) / D) / delta)
    out = np.empty_like(v)
    for c in range(3):
        out[L2C_IDX[face][c]] = L2C_SGN[face][c] * loc[c]
    return out


def cart_to_contra(v, face, alpha, beta):
    x, y, delta, C, D = _metric(alpha, beta)
    loc = [None] * 3
    for c in range(3):
        loc[C2L_IDX[face][c]] = C2L_SGN[face][c] * v[c]
    vz, vx, vy = loc
    return np.stack([(vz + x * vx + y * vy) / delta,
                     D / delta * (vx - x * vz),
                     C / delta * (vy - y * vz)])


def _raise(v, cth):
    out = v.copy()
    sth2 = 1. - cth * cth
    out[1] = v[1] / sth2 - v[2] * cth / sth2
    out[2] = -v[1] * cth / sth2 + v[2] / sth2
    return out


def _lower(v, cth):
    out = v.copy()
    out[1] = v[1] + v[2] * cth
    out[2] = v[2] + v[1] * cth
    return out


def _frame(face, alpha, beta):
    up = np.zeros((3,) + np.shape(alpha))
    up[0] = 1.
    up = contra_to_cart(up, face, alpha, beta)
    z, x, y = up[0], up[1], up[2]
    s = np.sqrt(x * x + y * y)
    pole = s == 0.
    safe = np.where(pole, 1., s)
    return x, y, z, s, np.where(pole, 1., x / safe), np.where(pole, 0., y / safe)


def _cart_to_local(v, fr):
    x, y, z, s, cphi, sphi = fr
    vz, vx, vy = v[0], v[1], v[2]
    horiz = vx * cphi + vy * sphi
    return np.stack([horiz * s + vz * z, horiz * z - vz * s, -vx * sphi + vy * cphi])


def _local_to_cart(v, fr):
    x, y, z, s, cphi, sphi = fr
    vr, vt, vp = v[0], v[1], v[2]
    horiz = vr * s + vt * z
    return np.stack([vr * z - vt * s, horiz * cphi - vp * sphi, horiz * sphi + vp * cphi])


def rotation(face, alpha, beta, to_global, cosine=None):
    """PanelRotation::matrix: m[out, in, ...] for the panel's components at
    (alpha, beta) to the geographic frame (to_global) or back; with a
    cosine the panel's components are covariant (conserved momenta)."""
    alpha, beta = np.broadcast_arrays(np.asarray(alpha, float), np.asarray(beta, float))
    fr = _frame(face, alpha, beta)
    m = np.empty((3, 3) + alpha.shape)
    for i in range(3):
        basis = np.zeros((3,) + alpha.shape)
        basis[i] = 1.
        if to_global:
            if cosine is not None:
                basis = _raise(basis, cosine)
            basis = _cart_to_local(contra_to_cart(basis, face, alpha, beta), fr)
        else:
            basis = cart_to_contra(_local_to_cart(basis, fr), face, alpha, beta)
            if cosine is not None:
                basis = _lower(basis, cosine)
        m[:, i] = basis
    return m


def apply(m, v):
    """v_out[i] = sum_j m[i, j] v[j] (cs_apply_velocity_transform_)."""
    return np.stack([m[i, 0] * v[0] + m[i, 1] * v[1] + m[i, 2] * v[2] for i in range(3)])


def geometry(n: int, r_in: float, dr: float = 1.0):
    """GnomonicEquiangleImpl::reset on one panel-sized block (nx2 = nx3 =
    n, nghost 3, one radial cell [r_in, r_in + dr]); arrays [k, j]."""
    import torch
    nc = n + 2 * NG
    d = (0.5 * math.pi) / n
    # CoordinateImpl::block_faces_: the global linspace with the ghosts
    xf = torch.linspace(-0.25 * math.pi - NG * d, 0.25 * math.pi + NG * d,
                        n + 2 * NG + 1, dtype=torch.float64).numpy()
    xv = 0.5 * (xf[:-1] + xf[1:])
    x, xff = np.tan(xv)[None, :], np.tan(xf)[None, :]
    y, yff = np.tan(xv)[:, None], np.tan(xf)[:, None]
    C, Cf = np.sqrt(1.0 + x * x), np.sqrt(1.0 + xff * xff)
    D, Df = np.sqrt(1.0 + y * y), np.sqrt(1.0 + yff * yff)
    g = {"x2f": xf, "x2v": xv}
    g["cos_c"] = -x * y / (C * D)
    g["sin_c"] = np.sqrt(1.0 + x * x + y * y) / (C * D)
    g["cos_f2"] = -xff * y / (Cf * D)
    g["sin_f2"] = np.sqrt(1.0 + xff * xff + y * y) / (Cf * D)
    g["cos_f3"] = -x * yff / (C * Df)
    g["sin_f3"] = np.sqrt(1.0 + x * x + yff * yff) / (C * Df)

    def arc(e, a, b):
        e2 = e * e
        return np.arccos((1. + e2 + a * b) /
                         (np.sqrt(1. + e2 + a * a) * np.sqrt(1. + e2 + b * b)))

    x1, x2 = np.tan(xf[:nc])[None, :], np.tan(xf[1:nc + 1])[None, :]
    y1, y2 = np.tan(xf[:nc])[:, None], np.tan(xf[1:nc + 1])[:, None]
    dx2f_ang = arc(y, x1, x2)
    dx2f_ang_face3 = arc(yff, x1, x2)
    dx3f_ang = arc(x, y1, y2)
    dx3f_ang_face2 = arc(xff, y1, y2)
    xc, yc = np.tan(xf)[None, :], np.tan(xf)[:, None]
    corner = np.arctan(xc * yc / np.sqrt(1. + xc * xc + yc * yc))
    solid = (corner[1:nc + 1, 1:nc + 1] - corner[1:nc + 1, 0:nc] -
             corner[0:nc, 1:nc + 1] + corner[0:nc, 0:nc])
    rm, rp = r_in, r_in + dr
    x1v = 0.5 * (rm + rp)
    g["radius"] = x1v
    g["area2"] = (x1v * dr) * dx3f_ang_face2
    g["area3"] = (x1v * dr) * dx2f_ang_face3
    g["vol"] = (dr * (rp * rp + rp * rm + rm * rm) / 3.0) * solid
    fx = g["area2"] * g["sin_f2"]
    fy = g["area3"] * g["sin_f3"]
    g["x_ov_rD"] = (fx[:, 1:nc + 1] - fx[:, 0:nc]) / g["vol"]
    g["y_ov_rC"] = (fy[1:nc + 1, :] - fy[0:nc, :]) / g["vol"]
    g["width2"] = x1v * dx2f_ang
    g["width3"] = x1v * dx3f_ang
    return g


def _xyz_to_ab(face, v):
    """cs_xyz_to_ab (src/coord/cubed_sphere_utils.cpp:53-76)."""
    vx, vy, vz = v
    a = {0: (vy, vx), 2: (-vy, -vx), 1: (-vx, vy), 4: (vx, -vy),
         3: (vy, vz), 5: (vy, -vz)}[face]
    b = {0: (vz, vx), 2: (vz, -vx), 1: (vz, vy), 4: (vz, -vy),
         3: (-vx, vz), 5: (vx, -vz)}[face]
    return math.atan2(*a), math.atan2(*b)


def usrc(N: int, nghost: int = NG) -> np.ndarray:
    """cs_build_ghost_usrc(N, nghost) for face 0, side L: [depth - 1, j]
    the source coordinate (cell-centre units) along the neighbour's edge."""
    d = math.pi / (2.0 * N)
    face_t, side_t = 0, SIDE_L
    nface, nside, rev = FACE_EDGES[face_t][side_t]
    out = np.empty((nghost, N))
    for depth in range(1, nghost + 1):
        for j in range(N):
            sgn = 1 if side_t in (SIDE_R, SIDE_T) else -1
            along = -math.pi / 4.0 + (j + 0.5) * d
            perp = sgn * (math.pi / 4.0 + (depth - 0.5) * d)
            if side_t in (SIDE_L, SIDE_R):
                at, bt = perp, along
            else:
                at, bt = along, perp
            X, Y, Z = face_xyz(face_t, np.float64(math.tan(at)), np.float64(math.tan(bt)))
            r = math.sqrt(X * X + Y * Y + Z * Z)
            a_s, b_s = _xyz_to_ab(nface, (X / r, Y / r, Z / r))
            ang = b_s if nside in (SIDE_L, SIDE_R) else a_s
            u = (ang + math.pi / 4.0) / d - 0.5
            if rev:
                u = (N - 1) - u
            out[depth - 1, j] = u
    return out


def _side_of(dy, dx):
    return {(0, -1): SIDE_L, (0, 1): SIDE_R, (-1, 0): SIDE_B, (1, 0): SIDE_T}[(dy, dx)]


OFFSETS = ((0, -1), (0, 1), (-1, 0), (1, 0))  # (dy, dx) of L, R, B, T


def _strip(n, dy, dx, exterior, margin):
    """(k, j) slices of a side's strip (MeshBlockImpl::part): nghost deep,
    interior or exterior, widened along the edge by margin."""
    ng = NG
    along = slice(ng - margin, ng + n + margin)
    if dx != 0:
        j = (slice(ng, 2 * ng) if dx < 0 else slice(n, n + ng)) if not exterior else \
            (slice(0, ng) if dx < 0 else slice(n + ng, n + 2 * ng))
        return along, j
    k = (slice(ng, 2 * ng) if dy < 0 else slice(n, n + ng)) if not exterior else \
        (slice(0, ng) if dy < 0 else slice(n + ng, n + 2 * ng))
    return k, along


def fill(u: np.ndarray, g) -> None:
    """The seam halo of u (6, 4, nc, nc), conserved, in place."""
    n = u.shape[-1] - 2 * NG
    margin = NG  # cs_interp_margin
    xv = g["x2v"]
    alpha = np.broadcast_to(xv[None, :], (n + 2 * NG, n + 2 * NG))
    beta = np.broadcast_to(xv[:, None], (n + 2 * NG, n + 2 * NG))
    cos = g["cos_c"]
    src = u.copy()  # every panel packs from the state before any unpack
    # serialize: the send buffer of every (panel, side)
    send = {}
    for q in range(6):
        for dy, dx in OFFSETS:
            my_side = _side_of(dy, dx)
            nb, nb_side, rev = FACE_EDGES[q][my_side]
            ks, js = _strip(n, dy, dx, False, margin)
            buf = src[q][:, ks, js].copy()              # (4, L3, L2)
            m = rotation(q, alpha[ks, js], beta[ks, js], True, cos[ks, js])
            buf[IVX:IVZ + 1] = apply(m, buf[IVX:IVZ + 1])
            trans = (my_side - 1.5) * (nb_side - 1.5) < 0
            flip = (my_side % 2) == (nb_side % 2)
            # the reference's tensors are (var, x3, x2, x1): its dims -3 / -2
            # are this array's -2 / -1
            if rev:   # along the edge
                buf = np.flip(buf, -1 if dy != 0 else -2)
            if flip:  # across the edge
                buf = np.flip(buf, -2 if dy != 0 else -1)
            if trans:
                buf = buf.transpose(0, 2, 1).reshape(buf.shape)
            send[(q, my_side)] = np.ascontiguousarray(buf)
    # deserialize: each panel's four sides
    us = usrc(n)
    for p in range(6):
        for dy, dx in OFFSETS:
            side = _side_of(dy, dx)
            q, q_side, _ = FACE_EDGES[p][side]
            ksw, jsw = _strip(n, dy, dx, True, margin)
            wide = u[p][:, ksw, jsw]
            # the raw copy into the wide landing zone (flat order)
            u[p][:, ksw, jsw] = send[(q, q_side)].reshape(wide.shape)
            wide = u[p][:, ksw, jsw].copy()
            # interp_ghost: linear along the edge from the wide strip
            if dy != 0:   # B / T: along x2 (dim -1 here), depth rows in x3
                ut = us if dy > 0 else us[::-1, :]
                u0f = np.floor(ut)
                x = ut - u0f
                i0 = u0f.astype(np.int64) + margin
                assert i0.min() >= margin and i0.max() + 1 <= margin + n - 1
                rows = np.arange(NG)[:, None]
                b0 = wide[:, rows, i0]
                b1 = wide[:, rows, i0 + 1]
                ghost = b0 + x[None] * (b1 - b0)
                kn, jn = _strip(n, dy, dx, True, 0)
            else:         # L / R: along x3, depth columns in x2
                ut = us.T if dx > 0 else us.T[:, ::-1]
                u0f = np.floor(ut)
                x = ut - u0f
                i0 = u0f.astype(np.int64) + margin
                assert i0.min() >= margin and i0.max() + 1 <= margin + n - 1
                cols = np.arange(NG)[None, :]
                b0 = wide[:, i0, cols]
                b1 = wide[:, i0 + 1, cols]
                ghost = b0 + x[None] * (b1 - b0)
                kn, jn = _strip(n, dy, dx, True, 0)
            # back to this panel's covariant momenta at its ghost cells
            m = rotation(p, alpha[kn, jn], beta[kn, jn], False, cos[kn, jn])
            ghost[IVX:IVZ + 1] = apply(m, ghost[IVX:IVZ + 1])
            # the wide zone's margin cells were only interpolation sources:
            # the narrow ghosts take the result, the margins keep the raw copy
            # (they are corner cells, which no stencil reads)
            u[p][:, kn, jn] = ghost


def _face_points(n, side, g):
    """(alpha, beta, cosine) of a side's n interior faces, along the edge."""
    xf, xv = g["x2f"], g["x2v"]
    I = slice(NG, NG + n)
    if side in (SIDE_L, SIDE_R):
        jf = NG if side == SIDE_L else NG + n
        return np.full(n, xf[jf]), xv[I], g["cos_f2"][I, jf]
    kf = NG if side == SIDE_B else NG + n
    return xv[I], np.full(n, xf[kf]), g["cos_f3"][kf, I]


def _matching(p, side, n):
    """The neighbour, its side and, per face of p's side (along index m),
    the along index of the same face on the neighbour's side."""
    q, q_side, rev = FACE_EDGES[p][side]
    m = np.arange(n)
    return q, q_side, (n - 1 - m) if rev else m


def seam_states_all(w2l, w2r, w3l, w3r, g):
    """Exterior-side states of every seam face from the neighbour's own
    interior-side state at the same face, velocities contra(q) -> Cartesian
    -> contra(p) at that point (hydro_forward.cpp:719-757 with the layout's
    kPrimitive transform: the geographic frame of one point cancels).
    Arrays: w2* (6, 4, n, n + 1) [k, face j], w3* (6, 4, n + 1, n) [face k, j]."""
    n = w2l.shape[2]
    orig = {2: (w2l.copy(), w2r.copy()), 3: (w3l.copy(), w3r.copy())}

    def side_state(arrs, side, which):
        """interior ('in') or exterior ('ex') state of a side's n faces."""
        (l2, r2), (l3, r3) = arrs[2], arrs[3]
        if side == SIDE_L:
            return (r2 if which == "in" else l2)[:, :, :, 0]
        if side == SIDE_R:
            return (l2 if which == "in" else r2)[:, :, :, n]
        if side == SIDE_B:
            return (r3 if which == "in" else l3)[:, :, 0, :]
        return (l3 if which == "in" else r3)[:, :, n, :]

    out = {2: (w2l, w2r), 3: (w3l, w3r)}
    for p in range(6):
        for side in range(4):
            q, q_side, mq = _matching(p, side, n)
            src = side_state(orig, q_side, "in")[q][:, mq]   # (4, n)
            aq, bq, _ = _face_points(n, q_side, g)
            aq, bq = aq[mq], bq[mq]
            ap, bp, _ = _face_points(n, side, g)
            v = src[IVX:IVZ + 1]
            cart = contra_to_cart(v, q, aq, bq)
            st = src.copy()
            st[IVX:IVZ + 1] = cart_to_contra(cart, p, ap, bp)
            dst = side_state(out, side, "ex")
            dst[p] = st


def reconcile(F2, F3, g):
    """reconcile_panel_seams on full face arrays F2 (6, 4, nc, nc + 1) and
    F3 (6, 4, nc + 1, nc), in place."""
    n = F2.shape[2] - 2 * NG
    I = slice(NG, NG + n)
    own = {}
    for p in range(6):
        for side in range(4):
            F = F2 if side < 2 else F3
            plane = {SIDE_L: NG, SIDE_R: NG + n, SIDE_B: NG, SIDE_T: NG + n}[side]
            own[(p, side)] = (F[p][:, I, plane] if side < 2 else F[p][:, plane, I]).copy()
    for p in range(6):
        for side in range(4):
            q, q_side, rev = FACE_EDGES[p][side]
            if p < q:
                continue  # the lower panel owns the seam
            a, b, c = _face_points(n, q_side, g)
            rows = own[(q, q_side)].copy()
            v = _raise(rows[IVX:IVZ + 1], c)
            rows[IVX:IVZ + 1] = contra_to_cart(v, q, a, b)
            if rev:
                rows = rows[:, ::-1]
            if (side % 2) == (q_side % 2):
                rows = -rows
            a, b, c = _face_points(n, side, g)
            v = cart_to_contra(rows[IVX:IVZ + 1], p, a, b)
            rows[IVX:IVZ + 1] = _lower(v, c)
            plane = {SIDE_L: NG, SIDE_R: NG + n, SIDE_B: NG, SIDE_T: NG + n}[side]
            if side < 2:
                F2[p][:, I, plane] = rows
            else:
                F3[p][:, plane, I] = rows
