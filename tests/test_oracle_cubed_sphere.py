"""The cubed-sphere geometry and seam tables, and the oracle that checks the
GPU path: solid angles close the sphere, the seam halo reproduces smooth
scalar and vector (solid-body rotation) fields to second order, the oracle's
shallow-roe is the reference kernel's bit for bit, and the oracle conserves
mass to roundoff and keeps a lake at rest."""
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


def halo_errors(n):
    g = cs.geometry(n, 6.371e6)
    from oracle.cubed_sphere import CubedSphere
    o = CubedSphere(n, g, cs.ghost_table(n, g), cs.seam_table(n, g), cs.RK3, 0.9)
    f, m2, m3 = fields(n, g)
    u = np.zeros((6, 4, n + 2 * NG, n + 2 * NG))
    u[:, 0], u[:, 2], u[:, 3] = f, m2, m3
    t = o.gt
    d = t[:, 0].astype(int)
    u2 = u.copy()
    o.fill(u2)
    flat = lambda a: a.transpose(1, 0, 2, 3).reshape(4, -1)
    e = np.abs(flat(u2)[:, d] - flat(u)[:, d])
    return e[0].max(), max(e[2].max(), e[3].max())


def test_solid_angles_close_the_sphere():
    for n in (8, 24):
        g = cs.geometry(n, 1.0)
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
    n = 12
    g = cs.geometry(n, 6.371e6)
    return CubedSphere(n, g, cs.ghost_table(n, g), cs.seam_table(n, g), cs.RK3, 0.9)


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
    g = cs.geometry(n, 6.371e6)
    gt, st = cs.ghost_table(n, g), cs.seam_table(n, g)
    roe = CubedSphere(n, g, gt, st, cs.RK3, 0.9)
    hllc = CubedSphere(n, g, gt, st, cs.RK3, 0.9, riemann="hllc")
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
