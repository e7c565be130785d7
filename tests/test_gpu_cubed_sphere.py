"""The cubed-sphere stage on the GPU (six panels, one handle) against the
oracle, whose geometry and seam exchanges restate the reference's own
routines (oracle/cs_seams.py): the seam halo, the stage in FP64 at relative
L2 1e-12 (n = 16, and the benchmark's 6 x 96^2 over 3 steps), mass conserved
to roundoff, a lake at rest, and the FP32 state against the FP64 oracle."""
import numpy as np
import pytest
import torch

from snapy_gb300 import cubed_sphere as cs

pytestmark = pytest.mark.gpu

NG = cs.NG


def oracle_sphere(n, riemann="shallow-roe"):
    from oracle.cubed_sphere import CubedSphere
    return CubedSphere(n, cs.RK3, 0.9, riemann=riemann)


def ghost_mask(n):
    nc = n + 2 * NG
    m = np.zeros((nc, nc), dtype=bool)
    I = slice(NG, NG + n)
    m[I, :NG] = m[I, NG + n:] = m[:NG, I] = m[NG + n:, I] = True
    return m


def errors(got, want):
    """Relative L2 per field over the interior; the radial momentum row (0
    on both sides up to the reference's round-off) against the tangential
    momenta's norm."""
    e = rel_l2(got, want)
    e[1] = np.linalg.norm(got[:, 1] - want[:, 1]) / np.linalg.norm(want[:, 2:])
    return e


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
    m = ghost_mask(n)
    assert np.abs(got[:, 0][:, m] - u[:, 0][:, m]).max() <= 1e-15 * 9500.
    sc = np.abs(u[:, 2:][:, :, m]).max()
    assert np.abs(got[:, 1:][:, :, m] - u[:, 1:][:, :, m]).max() <= 1e-13 * sc


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
        err = errors(interior(sp.state().cpu().numpy(), n), interior(u, n))
        assert err.max() <= 1e-12, (step, err)


def test_stage_parity_fp64_6x96(cuda):
    """The benchmark's grid, 6 panels of 96 x 96, seeded bump: 3 RK3 steps
    of the FP64 GPU path against the oracle at relative L2 1e-12 per field,
    mass conserved to round-off."""
    n = 96
    o = oracle_sphere(n)
    u = cs.bump(n, seed=20261206)
    sp = cs.SphereSW(n, dtype=torch.float64, device=cuda, graphs=False)
    sp.initialize(u)
    o.fill(u)
    m0 = o.mass(u)
    u0 = np.zeros_like(u)
    for step in range(3):
        dt = float(sp.max_dt().item())
        assert dt == pytest.approx(o.max_dt(u), rel=1e-15)
        sp.step(dt)
        for s in range(3):
            o.stage(u, u0, dt, s)
        err = errors(interior(sp.state().cpu().numpy(), n), interior(u, n))
        assert err.max() <= 1e-12, (step, err)
    assert abs(sp.mass() / m0 - 1) < 1e-13


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


def field_errors(got, want):
    """A step field's relative L2: the Phi row alone, and the three momentum
    rows together (the radial row is round-off on both sides, and a
    transverse row can be small beside the normal one)."""
    e0 = np.linalg.norm(got[:, 0] - want[:, 0]) / np.linalg.norm(want[:, 0])
    e1 = np.linalg.norm(got[:, 1:] - want[:, 1:]) / np.linalg.norm(want[:, 1:])
    return np.array([e0, e1])


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_step_fields_and_budget_against_oracle(cuda, dtype):
    """The FluxRegister's step fields of the six panels (both directions,
    every interior face, the seam faces single-valued) and the budget's row
    totals against the oracle: FP64 at 1e-12 (the field update is one fused
    multiply-add on the device, two roundings in the oracle); FP32 within
    1e-5 (its normal-momentum rows with phi_ref^2 / 2 added back); the
    total of Phi conserved to round-off."""
    n = 16
    o = oracle_sphere(n)
    u = cs.bump(n, seed=5, width=0.4)
    sp = cs.SphereSW(n, dtype=dtype, device=cuda, graphs=False)
    sp.initialize(u)
    S2 = sp.request_step_field(2)
    S3 = sp.request_step_field(3)
    o.fill(u)
    So = o.request_step_fields()
    t0 = sp.budget_totals().cpu().numpy()
    assert np.allclose(t0, o.budget_totals(u), rtol=1e-13 if dtype == torch.float64 else 1e-6)
    u0 = np.zeros_like(u)
    tol = 1e-12 if dtype == torch.float64 else 1e-5
    for step in range(3):
        dt = float(o.max_dt(u))
        sp.step(dt)
        for s in range(3):
            o.stage(u, u0, dt, s)
        for got, want in ((S2, So[2]), (S3, So[3])):
            e = field_errors(got.cpu().numpy(), want)
            assert e.max() <= tol, (step, e)
    print(f"\n{dtype}: step fields vs oracle, rel L2 (Phi row, momentum rows) "
          f"{field_errors(S2.cpu().numpy(), So[2])} {field_errors(S3.cpu().numpy(), So[3])}")
    t1 = sp.budget_totals().cpu().numpy()
    assert abs(t1[0] / t0[0] - 1) <= (1e-13 if dtype == torch.float64 else 1e-6)
    assert np.allclose(t1, o.budget_totals(u), rtol=tol, atol=tol * np.abs(t1).max())
