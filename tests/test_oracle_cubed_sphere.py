"""The cubed-sphere geometry and seam tables, and the oracle that checks the
GPU path.  The oracle's geometry and seam exchanges restate the reference's
own routines (oracle/cs_seams.py); the product's host tables are checked
against them here: the geometry bit for bit, the ghost table (its device
formula emulated) to round-off.  Also: solid angles close the sphere, the
seam halo reproduces smooth scalar and vector (solid-body rotation) fields to
second order, the oracle's shallow-roe is the reference kernel's bit for bit,
and the oracle conserves mass to roundoff and keeps a lake at rest."""
import math
import os

import numpy as np
import pytest

from snapy_gb300 import cubed_sphere as cs

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "shallow_roe.npz")
NG = cs.NG


def fields(n, g):
    """A smooth scalar and the covariant momentum of a solid-body rotation
    at every padded cell centre of the six panels."""
    nc = n + 2 * NG
    x2v = g["x2v"]
    B, A = np.meshgrid(x2v, x2v, indexing="ij")
    f = np.zeros((6, nc, nc))
    m2, m3 = np.zeros_like(f), np.zeros_like(f)
    om = np.array([0.3, -0.5, 0.8])
    for p in range(6):
        P = cs.point(p, A, B)
        f[p] = P @ np.array([1., 2., 3.]) + P[..., 0] * P[..., 1]
        V = np.cross(om, P)
        ta, tb = cs.tangents(p, A, B)
        m2[p], m3[p] = (V * ta).sum(-1), (V * tb).sum(-1)
    return f, m2, m3


def ghost_mask(n):
    """The seam ghost cells of a padded panel (the four strips, no
    corners)."""
    nc = n + 2 * NG
    m = np.zeros((nc, nc), dtype=bool)
    I = slice(NG, NG + n)
    m[I, :NG] = m[I, NG + n:] = m[:NG, I] = m[NG + n:, I] = True
    return m


def emulate_ghost_table(u, gt):
    """The device seam-halo gather (cs_ghost_kernel) on the host, in FP64:
    Phi and the radial momentum interpolated, the tangential pair through
    the table's frames."""
    nc = u.shape[-1]
    flat = u.transpose(1, 0, 2, 3).reshape(4, -1)
    d, s0, s1 = (gt[:, q].astype(np.int64) for q in range(3))
    x = gt[:, 3]
    for v in (0, 1):
        a, b = flat[v, s0], flat[v, s1]
        flat[v, d] = a + x * (b - a)

    def glob(idx, c, ta, tb):
        m2, m3 = flat[2, idx], flat[3, idx]
        s2 = 1. - c * c
        v2 = m2 / s2 - m3 * c / s2
        v3 = -m2 * c / s2 + m3 / s2
        return [ta[:, q] * v2 + tb[:, q] * v3 for q in range(3)]

    V0 = glob(s0, gt[:, 4], gt[:, 5:8], gt[:, 8:11])
    V1 = glob(s1, gt[:, 11], gt[:, 12:15], gt[:, 15:18])
    V = [V0[q] + x * (V1[q] - V0[q]) for q in range(3)]
    ta, tb = gt[:, 18:21], gt[:, 21:24]
    flat[2, d] = (V[0] * ta[:, 0] + V[1] * ta[:, 1]) + V[2] * ta[:, 2]
    flat[3, d] = (V[0] * tb[:, 0] + V[1] * tb[:, 1]) + V[2] * tb[:, 2]
    u[:] = flat.reshape(4, 6, nc, nc).transpose(1, 0, 2, 3)


def halo_errors(n):
    from oracle.cubed_sphere import CubedSphere
    o = CubedSphere(n, cs.RK3, 0.9)
    f, m2, m3 = fields(n, o.g)
    u = np.zeros((6, 4, n + 2 * NG, n + 2 * NG))
    u[:, 0], u[:, 2], u[:, 3] = f, m2, m3
    u2 = u.copy()
    o.fill(u2)
    m = ghost_mask(n)
    e = np.abs(u2[:, :, m] - u[:, :, m])
    return e[:, 0].max(), max(e[:, 2].max(), e[:, 3].max())


def test_geometry_is_the_references():
    """The product's host geometry equals the restatement of
    GnomonicEquiangleImpl::reset bit for bit."""
    from oracle import cs_seams as R
    for n in (8, 24, 96):
        gp, go = cs.geometry(n, 6.371e6), R.geometry(n, 6.371e6)
        for k in ("cos_c", "sin_c", "cos_f2", "sin_f2", "cos_f3", "sin_f3",
                  "area2", "area3", "vol", "x_ov_rD", "y_ov_rC", "width2",
                  "width3"):
            assert np.array_equal(gp[k], go[k]), (n, k)


@pytest.mark.parametrize("n", [8, 24, 96])
def test_ghost_table_is_the_references_seam_fill(n):
    """The product's ghost table, applied as the device applies it, equals
    the restated reference seam exchange (serialize, flips, interp_ghost,
    the geographic-frame transport) to round-off on a random state."""
    from oracle import cs_seams as R
    rng = np.random.default_rng(n)
    u = np.zeros((6, 4, n + 2 * NG, n + 2 * NG))
    u[:, 0] = 9000. + 500. * rng.random(u[:, 0].shape)
    u[:, 2:] = 1e4 * rng.normal(size=u[:, 2:].shape)
    a, b = u.copy(), u.copy()
    emulate_ghost_table(a, cs.ghost_table(n, cs.geometry(n, 6.371e6)))
    R.fill(b, R.geometry(n, 6.371e6))
    m = ghost_mask(n)
    assert np.abs(a[:, 0][:, m] - b[:, 0][:, m]).max() <= 1e-15 * 9500.
    sc = np.abs(b[:, 2:][:, :, m]).max()
    for v in (1, 2, 3):  # the radial row carries the reference's round-off
        assert np.abs(a[:, v][:, m] - b[:, v][:, m]).max() <= 1e-13 * sc, v


def test_solid_angles_close_the_sphere():
    from oracle import cs_seams as R
    for n in (8, 24):
        for g in (cs.geometry(n, 1.0), R.geometry(n, 1.0)):
            om = g["vol"][NG:NG + n, NG:NG + n].sum() * 6 / ((2.0 ** 3 - 1.0) / 3.0)
            assert abs(om / (4 * math.pi) - 1) < 1e-13


def test_seam_halo_is_second_order():
    es8, ev8 = halo_errors(8)
    es32, ev32 = halo_errors(32)
    assert es32 < es8 / 10 and ev32 < ev8 / 10
    assert es32 < 2e-3 and ev32 < 5e-4


def test_seam_faces_pair_up():
    n = 8
    g = cs.geometry(n, 1.0)
    st = cs.seam_table(n, g)
    # 12 seams, one non-owning side each, n faces
    assert st.shape[0] == 12 * n
    assert set(np.unique(st[:, 4])) <= {-1.0, 1.0}


def test_oracle_shallow_roe_is_the_reference_kernel(oracle):
    d = np.load(GOLDEN)
    L = oracle.lib()
    for i, dim in enumerate(d["dims"]):
        wl, wr = np.ascontiguousarray(d["wl"]), np.ascontiguousarray(d["wr"])
        f = np.zeros_like(wl)
        L.og_shallow_roe_batch(oracle.ptr(wl.ravel()), oracle.ptr(wr.ravel()),
                               len(wl), int(dim), oracle.ptr(f.ravel()))
        assert np.array_equal(f, d["flux"][i])


@pytest.fixture
def sphere():
    from oracle.cubed_sphere import CubedSphere
    return CubedSphere(12, cs.RK3, 0.9)


def test_oracle_conserves_mass(sphere):
    u = cs.bump(sphere.n, seed=3, width=0.5)
    sphere.fill(u)
    u0 = np.zeros_like(u)
    m0 = sphere.mass(u)
    for _ in range(4):
        dt = sphere.max_dt(u)
        for s in range(3):
            sphere.stage(u, u0, dt, s)
    assert abs(sphere.mass(u) / m0 - 1) < 1e-13
    assert np.abs(u[:, 2:, NG:-NG, NG:-NG]).max() > 1.0  # it moved


def test_oracle_lake_at_rest(sphere):
    n = sphere.n
    u = np.zeros((6, 4, n + 2 * NG, n + 2 * NG))
    u[:, 0, NG:NG + n, NG:NG + n] = 9810.
    sphere.fill(u)
    u0 = np.zeros_like(u)
    for _ in range(3):
        dt = sphere.max_dt(u)
        for s in range(3):
            sphere.stage(u, u0, dt, s)
    assert np.abs(u[:, 1:, NG:-NG, NG:-NG]).max() < 1e-8


def test_hllc_is_close_to_shallow_roe_and_conservative():
    """The shallow-water HLLC has no reference kernel: it is pinned to the
    reference's shallow-roe solution (relative L2 1e-3 after a short run),
    exact mass conservation and the lake at rest."""
    from oracle.cubed_sphere import CubedSphere
    n = 16
    roe = CubedSphere(n, cs.RK3, 0.9)
    hllc = CubedSphere(n, cs.RK3, 0.9, riemann="hllc")
    u2 = cs.bump(n, seed=4, width=0.5)
    m0 = hllc.mass(u2)
    # the same dt sequence for both
    u1 = cs.bump(n, seed=4, width=0.5)
    roe.fill(u1)
    u2 = u1.copy()
    z1, z2 = np.zeros_like(u1), np.zeros_like(u1)
    for _ in range(5):
        dt = roe.max_dt(u1)
        for s in range(3):
            roe.stage(u1, z1, dt, s)
            hllc.stage(u2, z2, dt, s)
    I = slice(NG, NG + n)
    a, b = u2[:, 0, I, I], u1[:, 0, I, I]
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-3
    assert abs(hllc.mass(u2) / m0 - 1) < 1e-13
    lake = np.zeros_like(u1)
    lake[:, 0, I, I] = 9810.
    hllc.fill(lake)
    for _ in range(3):
        dt = hllc.max_dt(lake)
        for s in range(3):
            hllc.stage(lake, z2, dt, s)
    assert np.abs(lake[:, 1:, I, I]).max() < 1e-8


@pytest.mark.parametrize("n", [8, 24])
def test_seam_state_table_is_the_references_face_state_sync(n):
    """The product's seam face-state table, applied as the seam pass applies
    it (the neighbour's own interior-side state at its side and along index,
    its velocities mapped at the shared face), equals the restated
    cross-panel face-state sync to round-off."""
    from oracle import cs_seams as R
    from oracle.cubed_sphere import CubedSphere
    o = CubedSphere(n, cs.RK3, 0.9)
    u = cs.bump(n, seed=11, width=0.5)
    rng = np.random.default_rng(3)
    u[:, 2:, NG:NG + n, NG:NG + n] += 1e3 * rng.normal(size=(6, 2, n, n))
    o.fill(u)
    w = o.cons2prim(u)
    w2l, w2r = o._states(w, 2)
    w3l, w3r = o._states(w, 1)
    # each side's interior-side states before the sync (L / B: the right
    # state, R / T: the left), per panel (4, n)
    inner = {0: lambda q: w2r[q][:, :, 0].copy(), 1: lambda q: w2l[q][:, :, n].copy(),
             2: lambda q: w3r[q][:, 0, :].copy(), 3: lambda q: w3l[q][:, n, :].copy()}
    before = {(q, si): inner[si](q) for q in range(6) for si in range(4)}
    R.seam_states_all(w2l, w2r, w3l, w3r, o.g)
    tab = cs.seam_state_table(n).reshape(6, 4, n, cs.SEAM_STATE_STRIDE)
    for p in range(6):
        for side in range(4):
            t = tab[p, side]
            q, qs, mq = (t[:, i].astype(np.int64) for i in range(3))
            we = np.stack([before[(int(q[m]), int(qs[m]))][:, mq[m]] for m in range(n)])
            M = t[:, 4:13].reshape(n, 3, 3)
            ext = we.copy()
            ext[:, 1:] = np.einsum("mab,mb->ma", M, we[:, 1:])
            want = {0: w2l[p][:, :, 0], 1: w2r[p][:, :, n],
                    2: w3l[p][:, 0, :], 3: w3r[p][:, n, :]}[side].T
            assert np.abs(ext[:, 0] - want[:, 0]).max() <= 1e-15 * np.abs(want[:, 0]).max()
            sc = np.abs(want[:, 2:]).max()
            assert np.abs(ext[:, 1:] - want[:, 1:]).max() <= 1e-13 * sc, (p, side)


def test_seam_table_is_the_references_reconcile():
    """The product's seam flux table, applied as cs_seam_flux_kernel applies
    it, equals the restated reconcile_panel_seams (owner copy through the
    Cartesian frame) to round-off on random face fluxes."""
    from oracle import cs_seams as R
    n = 12
    nc = n + 2 * NG
    rng = np.random.default_rng(5)
    F2 = rng.normal(size=(6, 4, nc, nc + 1))
    F3 = rng.normal(size=(6, 4, nc + 1, nc))
    F2[:, 1] = F3[:, 1] = 0.0  # no radial momentum flux in shallow water
    a2, a3 = F2.copy(), F3.copy()
    f2 = a2.transpose(1, 0, 2, 3).reshape(4, -1)
    f3 = a3.transpose(1, 0, 2, 3).reshape(4, -1)
    src = {2: f2.copy(), 3: f3.copy()}
    for row in cs.seam_table(n, cs.geometry(n, 6.371e6)):
        dd, di, sd, si = int(row[0]), int(row[1]), int(row[2]), int(row[3])
        sign, c = row[4], row[5]
        ta_s, tb_s, ta_d, tb_d = row[6:9], row[9:12], row[12:15], row[15:18]
        s, dst = src[sd], (f2 if dd == 2 else f3)
        m2, m3 = s[2, si], s[3, si]
        s2 = 1. - c * c
        v2, v3 = m2 / s2 - m3 * c / s2, -m2 * c / s2 + m3 / s2
        V = ta_s * v2 + tb_s * v3
        dst[0, di] = sign * s[0, si]
        dst[1, di] = sign * s[1, si]
        dst[2, di] = sign * (V @ ta_d)
        dst[3, di] = sign * (V @ tb_d)
    a2 = f2.reshape(4, 6, nc, nc + 1).transpose(1, 0, 2, 3)
    a3 = f3.reshape(4, 6, nc + 1, nc).transpose(1, 0, 2, 3)
    b2, b3 = F2.copy(), F3.copy()
    R.reconcile(b2, b3, R.geometry(n, 6.371e6))
    for a, b in ((a2, b2), (a3, b3)):
        assert np.abs(a[:, 0] - b[:, 0]).max() == 0.0
        assert np.abs(a[:, 1:] - b[:, 1:]).max() <= 1e-13 * np.abs(b[:, 2:]).max()
