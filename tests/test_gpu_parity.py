"""FP64 CUDA stage against the CPU oracle (the reference algorithm restated).

Both sides get the same initial state and the same dt sequence; every field
must agree within relative L2 1e-12 (the parity bar; the FP64 kernels are
built without contraction, so agreement is normally bitwise)."""
import numpy as np
import pytest
import torch

import snapy_gb300 as sg
from snapy_gb300 import problems

pytestmark = pytest.mark.gpu

TOL = 1e-12


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    out = []
    for v in range(a.shape[0]):
        den = np.linalg.norm(b[v])
        num = np.linalg.norm(a[v] - b[v])
        out.append(num / den if den > 0 else num)
    return np.array(out)


def deck(tmp_path, text):
    p = tmp_path / "deck.yaml"
    p.write_text(text)
    return sg.MeshBlockOptions.from_yaml(str(p))


def oracle_block(O, opts):
    return O.block_from_options(opts)


SOD = "snapy_gb300/decks/sod.yaml"


def test_sod_stage_by_stage(oracle, cuda):
    opts = sg.MeshBlockOptions.from_yaml(SOD)
    opts.execution = "eager"
    blk = sg.MeshBlock(opts).to(cuda)
    w = problems.sod(opts, cuda)
    vars = {"hydro_w": w}
    blk.initialize(vars)
    ob = oracle_block(oracle, opts)
    u = ob.initialize(w.cpu().numpy())
    np.testing.assert_array_equal(vars["hydro_u"].cpu().numpy(), u)
    for step in range(20):
        dt = blk.max_time_step(vars)
        dto = 0.4 * ob.max_dt(u)
        assert dt == dto
        for s in range(3):
            blk.forward(vars, dt, s)
            ob.stage(u, dt, s)
            err = rel_l2(vars["hydro_u"].cpu().numpy(), u)
            assert err.max() <= TOL, (step, s, err)
        assert blk.check_redo(vars) == 0


def test_sod_to_t02(oracle, cuda):
    opts = sg.MeshBlockOptions.from_yaml(SOD)
    blk = sg.MeshBlock(opts).to(cuda)
    w = problems.sod(opts, cuda)
    vars = {"hydro_w": w}
    blk.initialize(vars)
    ob = oracle_block(oracle, opts)
    u = ob.initialize(w.cpu().numpy())
    t = 0.0
    m0 = vars["hydro_u"][0, 0, 0, 3:-3].sum().item()
    while t < 0.2:
        dt = min(blk.max_time_step(vars), 0.2 - t)
        for s in range(3):
            blk.forward(vars, dt, s)
        assert blk.check_redo(vars) == 0
        ob.step(u, dt)
        t += dt
    err = rel_l2(vars["hydro_u"].cpu().numpy(), u)
    assert err.max() <= TOL, err
    m1 = vars["hydro_u"][0, 0, 0, 3:-3].sum().item()
    assert abs(m1 - m0) <= 1e-13 * m0
    rep = blk.execution_report()
    assert rep["replays"] > 0 and rep["captures"] == rep["graphs"]


DECK2D = """
geometry:
  type: cartesian
  bounds: {{x1min: 0., x1max: 1., x2min: 0., x2max: 1.5, x3min: 0., x3max: 1.}}
  cells: {{nx1: {nx1}, nx2: {nx2}, nx3: 1, nghost: 3}}
dynamics:
  equation-of-state: {{type: ideal-gas, gammad: 1.4}}
  reconstruct:
    vertical: {{type: weno5, scale: {scale}, shock: {shock}}}
    horizontal: {{type: weno5, scale: {scale}, shock: {shock}}}
  riemann-solver: {{type: {rs}}}
boundary-condition:
  external: {{x1-inner: {b1}, x1-outer: {b1}, x2-inner: {b2}, x2-outer: {b2}}}
integration: {{type: rk3, cfl: 0.6, execution: {ex}}}
"""


def smooth_state(opts, seed):
    c = opts.coord()
    g = torch.Generator().manual_seed(seed)
    x1 = torch.tensor(c.centers(1)).view(1, 1, -1)
    x2 = torch.tensor(c.centers(2)).view(1, -1, 1)
    w = torch.zeros((5, 1, c.nc2, c.nc1), dtype=torch.float64)
    a = torch.rand(6, generator=g, dtype=torch.float64)
    w[0] = 1.0 + 0.3 * torch.sin(6.0 * x1 + 3 * a[0]) * torch.cos(4.0 * x2 + a[1])
    w[1] = 0.4 * torch.sin(5.0 * x2 + a[2]) * torch.cos(3.0 * x1)
    w[2] = 0.3 * torch.cos(7.0 * x1 + a[3]) * torch.sin(2.0 * x2)
    w[3] = 0.1 * torch.sin(3 * x1 + 2 * x2)
    w[4] = 1.0 + 0.2 * torch.cos(4.0 * x1 + a[4]) + (x2 > 0.7) * 0.5
    return w


@pytest.mark.parametrize("rs,shock,scale,b1,b2", [
    ("lmars", "false", "false", "reflecting", "reflecting"),
    ("hllc", "true", "false", "periodic", "reflecting"),
    ("hllc", "false", "true", "extrapolation", "periodic"),
    ("lmars", "true", "false", "reflecting", "periodic"),
])
def test_2d_parity(oracle, cuda, tmp_path, rs, shock, scale, b1, b2):
    opts = deck(tmp_path, DECK2D.format(nx1=40, nx2=33, rs=rs, shock=shock,
                                        scale=scale, b1=b1, b2=b2, ex="eager"))
    blk = sg.MeshBlock(opts).to(cuda)
    w = smooth_state(opts, 3)
    vars = {"hydro_w": w.to(cuda)}
    blk.initialize(vars)
    ob = oracle_block(oracle, opts)
    u = ob.initialize(w.numpy())
    for step in range(6):
        dt = blk.max_time_step(vars)
        assert dt == 0.6 * ob.max_dt(u)
        for s in range(3):
            blk.forward(vars, dt, s)
            ob.stage(u, dt, s)
        err = rel_l2(vars["hydro_u"].cpu().numpy(), u)
        assert err.max() <= TOL, (step, err)


@pytest.mark.parametrize("tj", [1, 2, 5])
def test_tile_width_invariance(cuda, tmp_path, tj):
    """Any tile width gives the same bits (faces shared by two tiles are
    computed identically on both)."""
    text = DECK2D.format(nx1=24, nx2=37, rs="lmars", shock="false", scale="false",
                         b1="reflecting", b2="periodic", ex="eager")
    res = []
    for t in (0, tj):
        opts = deck(tmp_path, text)
        blk = sg.MeshBlock(opts, tj=t).to(cuda)
        vars = {"hydro_w": smooth_state(opts, 11).to(cuda)}
        blk.initialize(vars)
        for _ in range(3):
            dt = blk.max_time_step(vars)
            for s in range(3):
                blk.forward(vars, dt, s)
        res.append(vars["hydro_u"].clone())
    assert torch.equal(res[0], res[1])


def test_graph_equals_eager(cuda, tmp_path):
    out = {}
    for ex in ("eager", "cuda-graph"):
        opts = deck(tmp_path, DECK2D.format(nx1=32, nx2=32, rs="hllc", shock="true",
                                            scale="false", b1="reflecting",
                                            b2="reflecting", ex=ex))
        blk = sg.MeshBlock(opts).to(cuda)
        vars = {"hydro_w": smooth_state(opts, 5).to(cuda)}
        blk.initialize(vars)
        for _ in range(5):
            dt = blk.max_time_step(vars)
            for s in range(3):
                blk.forward(vars, dt, s)
            assert blk.check_redo(vars) == 0
        out[ex] = vars["hydro_u"].clone()
        if ex == "cuda-graph":
            assert blk.execution_report()["replays"] >= 6
    assert torch.equal(out["eager"], out["cuda-graph"])


def test_redo_restores_step(cuda, tmp_path):
    """A NaN planted in the state (on the host side) makes check_redo reject
    the step and restore the stage-0 state (MeshBlockImpl::apply_redo)."""
    opts = deck(tmp_path, DECK2D.format(nx1=16, nx2=16, rs="lmars", shock="false",
                                        scale="false", b1="reflecting",
                                        b2="reflecting", ex="eager"))
    blk = sg.MeshBlock(opts).to(cuda)
    vars = {"hydro_w": smooth_state(opts, 1).to(cuda)}
    blk.initialize(vars)
    u_start = vars["hydro_u"].clone()
    dt = blk.max_time_step(vars)
    blk.forward(vars, dt, 0)
    vars["hydro_u"][0, 0, 8, 8] = float("nan")
    blk.forward(vars, dt, 1)
    blk.forward(vars, dt, 2)
    assert blk.check_redo(vars) == 1
    assert torch.equal(vars["hydro_u"], u_start)
    assert blk.intg.current_redo == 1
    dt2 = blk.max_time_step(vars)
    assert dt2 == pytest.approx(dt / 2, rel=1e-15)


STRAKA = "snapy_gb300/decks/straka_noimplicit.yaml"


@pytest.mark.parametrize("nu,cov", [(75.0, True), (0.0, False)])
def test_straka_explicit_parity(oracle, cuda, nu, cov):
    """Gravity (well-balanced x1 reference, face-form gravity work),
    viscosity and the x2 covariance row: a 64 x 48 window of the Straka
    density current at 50 m, 8 steps of fixed dt."""
    opts = sg.MeshBlockOptions.from_yaml(STRAKA)
    c = opts.coord()
    c.nx1, c.nx2 = 48, 64
    c.x1max, c.x2max = 48 * 50.0, 64 * 50.0
    opts.hydro().diffusion.nu_iso = nu
    opts.hydro().flux_covariance = cov
    opts.execution = "eager"
    blk = sg.MeshBlock(opts).to(cuda)
    w = problems.straka(opts, "cpu", xc=1600.0, zc=1200.0, xr=800.0, zr=600.0)
    vars = {"hydro_w": w.to(cuda)}
    blk.initialize(vars)
    ob = oracle_block(oracle, opts)
    u = ob.initialize(w.numpy())
    np.testing.assert_array_equal(vars["hydro_u"].cpu().numpy(), u)
    for step in range(8):
        dt = blk.max_time_step(vars)
        assert dt == pytest.approx(0.9 * ob.max_dt(u), rel=1e-15)
        for s in range(3):
            blk.forward(vars, dt, s)
            ob.stage(u, dt, s)
        err = rel_l2(vars["hydro_u"].cpu().numpy(), u)
        assert err.max() <= TOL, (step, err)


def test_straka_rest_state_balanced(cuda):
    """An isentropic atmosphere at rest keeps its momentum at round-off: the
    well-balanced x1 reference cancels the hydrostatic pressure gradient."""
    opts = sg.MeshBlockOptions.from_yaml(STRAKA)
    c = opts.coord()
    c.nx1, c.nx2 = 64, 32
    c.x1max, c.x2max = 64 * 50.0, 32 * 50.0
    blk = sg.MeshBlock(opts).to(cuda)
    vars = {"hydro_w": problems.straka(opts, cuda, dT=0.0)}
    blk.initialize(vars)
    for _ in range(10):
        blk.step(vars, 0.1)
    w = blk.prim()
    assert w[1:4].abs().max().item() < 1e-9


STRAKA_VIC = "snapy_gb300/decks/straka.yaml"


def test_straka_implicit_parity(oracle, cuda):
    """The full Straka stage with the vertical implicit correction (scheme 9:
    5x5 blocks, Woodbury wall rows, redistribution, gravity-work remainder)
    against the oracle on a 48 x 40 window, 6 steps."""
    opts = sg.MeshBlockOptions.from_yaml(STRAKA_VIC)
    c = opts.coord()
    c.nx1, c.nx2 = 48, 40
    c.x1max, c.x2max = 48 * 50.0, 40 * 50.0
    opts.execution = "eager"
    blk = sg.MeshBlock(opts).to(cuda)
    w = problems.straka(opts, "cpu", xc=1000.0, zc=1200.0, xr=800.0, zr=600.0)
    vars = {"hydro_w": w.to(cuda)}
    blk.initialize(vars)
    ob = oracle_block(oracle, opts)
    u = ob.initialize(w.numpy())
    for step in range(6):
        dt = blk.max_time_step(vars)
        assert dt == pytest.approx(0.9 * ob.max_dt(u), rel=1e-15)
        for s in range(3):
            blk.forward(vars, dt, s)
            ob.stage(u, dt, s)
        assert blk.check_redo(vars) == 0
        err = rel_l2(vars["hydro_u"].cpu().numpy(), u)
        assert err.max() <= TOL, (step, err)


def test_implicit_rest_state_balanced(cuda):
    opts = sg.MeshBlockOptions.from_yaml(STRAKA_VIC)
    c = opts.coord()
    c.nx1, c.nx2 = 64, 24
    c.x1max, c.x2max = 64 * 50.0, 24 * 50.0
    blk = sg.MeshBlock(opts).to(cuda)
    vars = {"hydro_w": problems.straka(opts, cuda, dT=0.0)}
    blk.initialize(vars)
    for _ in range(10):
        blk.step(vars, 0.1)
    assert blk.prim()[1:4].abs().max().item() < 1e-9


def test_implicit_wide_batch_parity(oracle, cuda):
    """A block with columns enough to fill every SM sub-partition (20480)
    takes the thread-per-column finish of the implicit solve: the same
    operations in the same order, so parity holds as for the warp form."""
    opts = sg.MeshBlockOptions.from_yaml(STRAKA_VIC)
    c = opts.coord()
    c.nx1, c.nx2 = 6, 20480
    c.x1max, c.x2max = 6 * 50.0, 20480 * 50.0
    opts.execution = "eager"
    blk = sg.MeshBlock(opts).to(cuda)
    w = problems.straka(opts, "cpu", xc=5000.0, zc=150.0, xr=2000.0, zr=100.0)
    vars = {"hydro_w": w.to(cuda)}
    blk.initialize(vars)
    ob = oracle_block(oracle, opts)
    u = ob.initialize(w.numpy())
    for step in range(2):
        dt = blk.max_time_step(vars)
        for s in range(3):
            blk.forward(vars, dt, s)
            ob.stage(u, dt, s)
        assert blk.check_redo(vars) == 0
        err = rel_l2(vars["hydro_u"].cpu().numpy(), u)
        assert err.max() <= TOL, (step, err)
