"""3-D blocks (x3 faces by the x3 sweep, (x2, x3) columns of the implicit
solve) against the oracle: FP64 parity at relative L2 1e-12 with and without
the flux-covariance row, FP32 anomalies within 1e-5 of the FP64 oracle, and
an x3-uniform 3-D block equal bit for bit to its 2-D slice."""
import numpy as np
import pytest
import torch

import snapy_gb300 as sg
from snapy_gb300 import problems

pytestmark = pytest.mark.gpu

TOL = 1e-12
TOL32 = 1e-5


def rel_l2(a, b):
    out = []
    for v in range(a.shape[0]):
        den = np.linalg.norm(b[v])
        num = np.linalg.norm(a[v] - b[v])
        out.append(num / den if den > 0 else num)
    return np.array(out)


def conv_window(nx1, nx2, nx3, precision, implicit=True, dtheta=2.0, cov=True,
                nu=0.0):
    opts = sg.MeshBlockOptions.from_yaml("snapy_gb300/decks/convection3d.yaml")
    opts.hydro().flux_covariance = cov
    if nu:
        from snapy_gb300.options import DiffusionOptions
        opts.hydro().diffusion = DiffusionOptions(nu_iso=nu, raw={"nu_iso": nu})
    c = opts.coord()
    c.nx1, c.nx2, c.nx3 = nx1, nx2, nx3
    c.x1max, c.x2max, c.x3max = nx1 * 50.0, nx2 * 50.0, nx3 * 50.0
    opts.hydro().precision = precision
    opts.problem["dtheta"] = dtheta
    opts.problem["layer"] = 0.4
    if not implicit:
        opts.hydro().icorr = None
    opts.execution = "eager"
    return opts


def interior(opts, u):
    c = opts.coord()
    ng = c.nghost
    return u[:, ng:c.nc3 - ng, ng:c.nc2 - ng, ng:c.nc1 - ng]


@pytest.mark.parametrize("cov", [False, True])
@pytest.mark.parametrize("implicit", [False, True])
def test_3d_fp64_parity(oracle, cuda, implicit, cov):
    """With the covariance row (the reference's default, on x2 and x3
    faces) and without."""
    opts = conv_window(24, 12, 10, "float64", implicit, cov=cov)
    blk = sg.MeshBlock(opts).to(cuda)
    w = problems.convection3d(opts, "cpu", seed=11)
    vars = {"hydro_w": w.to(cuda)}
    blk.initialize(vars)
    ob = oracle.block_from_options(opts)
    u = ob.initialize(w.numpy())
    for step in range(3):
        dt = blk.max_time_step(vars)
        assert dt == pytest.approx(0.9 * ob.max_dt(u), rel=1e-14)
        for s in range(3):
            blk.forward(vars, dt, s)
            ob.stage(u, dt, s)
        assert blk.check_redo(vars) == 0
        err = rel_l2(vars["hydro_u"].cpu().numpy(), u)
        assert err.max() <= TOL, (step, err)


@pytest.mark.parametrize("implicit", [False, True])
def test_3d_viscosity_fp64_parity(oracle, cuda, implicit):
    """Viscosity on a 3-D block (nu_iso 75 m^2/s, the x1, x2 and x3 viscous
    fluxes with their shear terms) with the covariance row, against the
    oracle at 1e-12."""
    opts = conv_window(20, 12, 10, "float64", implicit, nu=75.0)
    blk = sg.MeshBlock(opts).to(cuda)
    w = problems.convection3d(opts, "cpu", seed=13)
    vars = {"hydro_w": w.to(cuda)}
    blk.initialize(vars)
    ob = oracle.block_from_options(opts)
    u = ob.initialize(w.numpy())
    for step in range(3):
        dt = blk.max_time_step(vars)
        assert dt == pytest.approx(opts.intg().cfl * ob.max_dt(u), rel=1e-14)
        for s in range(3):
            blk.forward(vars, dt, s)
            ob.stage(u, dt, s)
        assert blk.check_redo(vars) == 0
        err = rel_l2(vars["hydro_u"].cpu().numpy(), u)
        assert err.max() <= TOL, (step, err)


def test_3d_viscosity_fp32_against_fp64_oracle(oracle, cuda):
    opts = conv_window(20, 12, 10, "float32", True, nu=75.0)
    blk = sg.MeshBlock(opts).to(cuda)
    w = problems.convection3d(opts, "cpu", seed=17)
    vars = {"hydro_w": w.to(cuda)}
    blk.initialize(vars)
    ob = oracle.block_from_options(opts)
    u = ob.initialize(w.numpy())
    dt = 0.9 * ob.max_dt(u)
    for _ in range(10):
        blk.step(vars, dt)
        for s in range(3):
            ob.stage(u, dt, s)
    assert blk.check_redo(vars) == 0
    err = rel_l2(interior(opts, blk.total_u(vars).cpu().numpy()), interior(opts, u))
    assert err.max() <= TOL32, err


def test_3d_fp32_anomaly_against_fp64_oracle(oracle, cuda):
    opts = conv_window(24, 16, 12, "float32", True)
    blk = sg.MeshBlock(opts).to(cuda)
    w = problems.convection3d(opts, "cpu", seed=5)
    vars = {"hydro_w": w.to(cuda)}
    blk.initialize(vars)
    ob = oracle.block_from_options(opts)
    u = ob.initialize(w.numpy())
    dt = 0.9 * ob.max_dt(u)
    for _ in range(20):
        blk.step(vars, dt)
        for s in range(3):
            ob.stage(u, dt, s)
    assert blk.check_redo(vars) == 0
    got = blk.total_u(vars).cpu().numpy()
    err = rel_l2(interior(opts, got), interior(opts, u))
    print(f"\n3-D convection: FP32 anomaly vs FP64 oracle after 20 steps, "
          "rel L2 (rho, m1, m2, m3, E): " + " ".join(f"{e:.2e}" for e in err))
    assert err.max() <= TOL32, err


def test_3d_x3_uniform_equals_2d(cuda):
    o2 = conv_window(24, 12, 1, "float64", True)
    o2.bcnames = list(o2.bcnames[:4])
    o3 = conv_window(24, 12, 8, "float64", True)
    w3 = problems.convection3d(o3, "cpu", seed=3)
    c3 = o3.coord()
    w3 = w3[:, c3.nghost:c3.nghost + 1].expand(-1, c3.nc3, -1, -1).contiguous()
    w2 = w3[:, :1].contiguous()
    b2, b3 = sg.MeshBlock(o2).to(cuda), sg.MeshBlock(o3).to(cuda)
    v2, v3 = {"hydro_w": w2.to(cuda)}, {"hydro_w": w3.to(cuda)}
    b2.initialize(v2)
    b3.initialize(v3)
    for _ in range(3):
        dt = b2.max_time_step(v2)
        b2.step(v2, dt)
        b3.step(v3, dt)
    u2, u3 = v2["hydro_u"], v3["hydro_u"]
    for k in range(c3.nghost, c3.nc3 - c3.nghost):
        assert torch.equal(u3[:, k], u2[:, 0]), k
