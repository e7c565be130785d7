"""The cubed-sphere stage on the GPU (six panels, one handle) against the
oracle: the seam halo and the stage in FP64 at relative L2 1e-12 (the same
operations in the same order), mass conserved to roundoff, a lake at rest,
and the FP32 state against the FP64 oracle."""
import numpy as np
import pytest
import torch

from snapy_gb300 import cubed_sphere as cs

pytestmark = pytest.mark.gpu

NG = cs.NG


def oracle_sphere(n, riemann="shallow-roe"):
    from oracle.cubed_sphere import CubedSphere
    g = cs.geometry(n, 6.371e6)
    return CubedSphere(n, g, cs.ghost_table(n, g), cs.seam_table(n, g), cs.RK3, 0.9,
                       riemann=riemann)


def interior(u, n):
    return u[:, :, NG:NG + n, NG:NG + n]


def rel_l2(a, b):
    out = []
    for v in range(a.shape[1]):
        den = np.linalg.norm(b[:, v])
        num = np.linalg.norm(a[:, v] - b[:, v])
        out.append(num / den if den > 0 else num)
    return np.array(out)


def test_seam_fill_matches_oracle(cuda):
    n = 16
    o = oracle_sphere(n)
    rng = np.random.default_rng(1)
    u = np.zeros((6, 4, n + 2 * NG, n + 2 * NG))
    u[:, 0] = 9000. + 500. * rng.random(u[:, 0].shape)
    u[:, 2:] = 1e4 * rng.normal(size=u[:, 2:].shape)
    sp = cs.SphereSW(n, dtype=torch.float64, device=cuda)
    sp.initialize(u)
    o.fill(u)
    got = sp.state().cpu().numpy()
    d = o.gt[:, 0].astype(np.int64)
    flat = lambda a: a.transpose(1, 0, 2, 3).reshape(4, -1)
    assert np.array_equal(flat(got)[:, d], flat(u)[:, d])


@pytest.mark.parametrize("riemann", ["shallow-roe", "hllc"])
def test_stage_parity_fp64(cuda, riemann):
    n = 16
    o = oracle_sphere(n, riemann)
    u = cs.bump(n, seed=5, width=0.4)
    sp = cs.SphereSW(n, dtype=torch.float64, device=cuda, graphs=False,
                     riemann=riemann)
    sp.initialize(u)
    o.fill(u)
    u0 = np.zeros_like(u)
    for step in range(4):
        dt = float(sp.max_dt().item())
        assert dt == pytest.approx(o.max_dt(u), rel=1e-15)
        sp.step(dt)
        for s in range(3):
            o.stage(u, u0, dt, s)
        err = rel_l2(interior(sp.state().cpu().numpy(), n), interior(u, n))
        assert err[[0, 2, 3]].max() <= 1e-12, (step, err)


def test_mass_and_lake_at_rest(cuda):
    n = 24
    sp = cs.SphereSW(n, dtype=torch.float64, device=cuda)
    sp.initialize(cs.bump(n, seed=2))
    m0 = sp.mass()
    for _ in range(10):
        sp.step()
    assert abs(sp.mass() / m0 - 1) < 1e-13
    assert sp.replays >= 5
    lake = np.zeros((6, 4, n + 2 * NG, n + 2 * NG))
    lake[:, 0, NG:NG + n, NG:NG + n] = 9810.
    sp.initialize(lake)
    for _ in range(5):
        sp.step()
    assert sp.state()[:, 1:, NG:NG + n, NG:NG + n].abs().max().item() < 1e-8


@pytest.mark.parametrize("riemann", ["shallow-roe", "hllc"])
def test_fp32_against_fp64_oracle(cuda, riemann):
    """FP32 state storing Phi as an anomaly about the mean depth's
    geopotential, the pressure carried as an anomaly too: within the FP32
    bar (relative L2 1e-5) of the FP64 oracle."""
    n = 24
    o = oracle_sphere(n, riemann)
    u = cs.bump(n, seed=7, width=0.3)
    sp = cs.SphereSW(n, dtype=torch.float32, device=cuda, riemann=riemann)
    sp.initialize(u)
    o.fill(u)
    u0 = np.zeros_like(u)
    for _ in range(10):
        dt = o.max_dt(u)
        sp.step(dt)
        for s in range(3):
            o.stage(u, u0, dt, s)
    err = rel_l2(interior(sp.totals().cpu().numpy(), n), interior(u, n))
    print(f"\ncubed sphere n={n} ({riemann}): FP32 vs FP64 oracle after 10 steps, "
          f"rel L2 (Phi, m2, m3): {err[0]:.2e} {err[2]:.2e} {err[3]:.2e}")
    assert err[[0, 2, 3]].max() <= 1e-5
