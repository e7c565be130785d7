"""Passive scalars on the GPU (the scalar kernels through the C ABI) against
the oracle's restatement of ScalarImpl::forward and of the scalars' share of
the implicit solve's dry transfer: FP64 within 1e-12 of the oracle per
tracer and hydro field after 10 steps (Straka explicit and with the solve,
and a 1-D tube), the reference's own properties on the device (a uniform
ratio stays uniform, the tracer is conserved in a closed box), FP32 within
1e-5, without and with the flux-covariance row (the scalars' covariance
row and the shared positivity limiter), and the refusals of what is not
built."""
import copy

import numpy as np
import pytest
import torch

import snapy_gb300 as sg
from snapy_gb300 import problems
from snapy_gb300.ensemble import Ensemble
from snapy_gb300.options import DeckError

pytestmark = pytest.mark.gpu

INNER = (slice(None), slice(3, -3), slice(3, -3))


def straka(precision="float64", nx1=32, nx2=48, deck="straka_noimplicit.yaml",
           implicit_precision=None, cov=False):
    cfg = copy.deepcopy(sg.options.yaml_lite.load("snapy_gb300/decks/" + deck))
    cfg["scalar"] = {"nvar": 2, "names": ["uniform", "step"]}
    cfg["dynamics"]["flux-covariance"] = cov
    opts = sg.MeshBlockOptions.from_config(cfg)
    c = opts.coord()
    c.nx1, c.nx2, c.x1max, c.x2max = nx1, nx2, nx1 * 50.0, nx2 * 50.0
    opts.hydro().precision = precision
    if implicit_precision:
        opts.hydro().icorr.precision = implicit_precision
    opts.execution = "eager"
    opts.autotune = False
    return opts


def ratios(opts):
    c = opts.coord()
    i = np.arange(c.nc1)[None, None, :]
    shape = (c.nc3, c.nc2, c.nc1)
    return np.stack([np.full(shape, 0.37), np.where(i > 16, 2.0, 0.0) + np.zeros(shape)])


def run_pair(cuda, opts, oracle, nsteps=10):
    w = problems.straka(opts, "cpu", xc=1000.0, zc=1200.0, xr=800.0, zr=600.0)
    r = ratios(opts)
    blk = sg.MeshBlock(opts).to(cuda)
    vars = {"hydro_w": w.to(cuda), "scalar_r": torch.from_numpy(r).to(cuda)}
    blk.initialize(vars)
    ob = oracle.block_from_options(opts)
    u = ob.initialize(w.numpy())
    s = ob.set_scalars(u[0] * r)
    for _ in range(nsteps):
        dt = blk.max_time_step(vars)
        blk.step(vars, dt)
        assert blk.check_redo(vars) == 0
        ob.step(u, dt)
    return blk, vars, u, s


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("cov", [False, True])
@pytest.mark.parametrize("deck", ["straka_noimplicit.yaml", "straka.yaml"])
def test_fp64_scalars_against_oracle(oracle, cuda, deck, cov):
    """Explicit, and with the vertical implicit solve (the scalars' share of
    its dry transfer); without and with the flux-covariance row (the
    reference's default: the scalars' covariance row and the positivity
    limiter)."""
    opts = straka(deck=deck, cov=cov)
    blk, vars, u, s = run_pair(cuda, opts, oracle)
    got_s = vars["scalar_s"].double().cpu().numpy()
    got_u = blk.total_u(vars).double().cpu().numpy()
    es = [rel(got_s[v][INNER], s[v][INNER]) for v in range(2)]
    eu = [rel(got_u[v][INNER], u[v][INNER]) for v in range(5) if np.linalg.norm(u[v]) > 0]
    print(f"\n{deck} cov={cov}: FP64 scalars vs oracle, rel L2:", es,
          "hydro:", max(eu))
    assert max(es) <= 1e-12 and max(eu) <= 1e-12
    if cov:
        assert got_s[1][INNER].min() >= 0.0
    # the reference's properties, on the device's result
    ratio = got_s[0][INNER] / got_u[0][INNER]
    assert np.abs(ratio / 0.37 - 1).max() <= 1e-13
    vol = opts.coord().dx1 * opts.coord().dx2
    r0 = ratios(opts)
    w = problems.straka(opts, "cpu", xc=1000.0, zc=1200.0, xr=800.0, zr=600.0).numpy()
    for v in range(2):
        m0 = (w[0] * r0[v])[0, 3:-3, 3:-3].sum() * vol
        m = got_s[v][INNER].sum() * vol
        assert abs(m - m0) <= 1e-13 * abs(m0)


def test_fp64_scalar_tube_against_oracle(oracle, cuda):
    cfg = copy.deepcopy(sg.options.yaml_lite.load("snapy_gb300/decks/sod.yaml"))
    cfg["scalar"] = {"nvar": 1}
    opts = sg.MeshBlockOptions.from_config(cfg)
    opts.execution = "eager"
    opts.autotune = False
    w = problems.sod(opts, "cpu")
    c = opts.coord()
    x = np.linspace(0.0, 1.0, c.nc1)
    r = (0.5 + 0.4 * np.sin(6.0 * x))[None, None, None, :] * np.ones((1, 1, 1, c.nc1))
    blk = sg.MeshBlock(opts).to(cuda)
    vars = {"hydro_w": w.to(cuda), "scalar_r": torch.from_numpy(r).to(cuda)}
    blk.initialize(vars)
    ob = oracle.block_from_options(opts)
    u = ob.initialize(w.numpy())
    s = ob.set_scalars(u[0] * r)
    for _ in range(20):
        dt = blk.max_time_step(vars)
        blk.step(vars, dt)
        ob.step(u, dt)
    got = vars["scalar_s"].double().cpu().numpy()
    e = rel(got[0, 0, 0, 3:-3], s[0, 0, 0, 3:-3])
    print(f"\n1-D tube tracer vs oracle: rel L2 {e:.2e}")
    assert e <= 1e-12


@pytest.mark.parametrize("cov", [False, True])
@pytest.mark.parametrize("deck,ip", [("straka_noimplicit.yaml", None),
                                     ("straka.yaml", "float32")])
def test_fp32_scalars_against_fp64_oracle(oracle, cuda, deck, ip, cov):
    opts = straka("float32", deck=deck, implicit_precision=ip, cov=cov)
    blk, vars, u, s = run_pair(cuda, opts, oracle)
    got_s = vars["scalar_s"].double().cpu().numpy()
    es = [rel(got_s[v][INNER], s[v][INNER]) for v in range(2)]
    print(f"\n{deck}: FP32 scalars vs FP64 oracle, rel L2:", es)
    assert max(es) <= 1e-5


def test_graphs_and_redo_carry_the_scalars(cuda):
    """Captured steps give the eager result bit for bit, and a rejected step
    restores the scalars with the state (the buffer rotation)."""
    out = []
    for execution in ("eager", "cuda-graph"):
        opts = straka()
        opts.execution = execution
        w = problems.straka(opts, "cpu", xc=1000.0, zc=1200.0, xr=800.0, zr=600.0)
        blk = sg.MeshBlock(opts).to(cuda)
        vars = {"hydro_w": w.to(cuda),
                "scalar_r": torch.from_numpy(ratios(opts)).to(cuda)}
        blk.initialize(vars)
        for _ in range(4):
            blk.step(vars, blk.max_time_step(vars))
        out.append(vars["scalar_s"].clone())
    assert torch.equal(out[0], out[1])
    blk.batch.restore()
    blk._publish(vars)
    assert not torch.equal(vars["scalar_s"], out[1])


def test_scalar_refusals(cuda):
    cfg = copy.deepcopy(sg.options.yaml_lite.load("snapy_gb300/decks/straka.yaml"))
    cfg["scalar"] = {"nvar": 1, "upper-bound": 1.0}
    with pytest.raises(DeckError, match="upper-bound"):
        sg.MeshBlockOptions.from_config(cfg)
    opts = straka()
    blk = sg.MeshBlock(opts).to(cuda)
    w = problems.straka(opts, "cpu")
    with pytest.raises(RuntimeError, match="scalar_r"):
        blk.initialize({"hydro_w": w.to(cuda)})


def test_ensemble_member_alone_equals_in_the_batch(cuda):
    """Two members of uneven size with tracers, one with the implicit solve:
    each member's tracers and state after 5 steps in the batch equal the
    member stepped alone as a MeshBlock, bit for bit."""
    members = [straka(nx1=32, nx2=48), straka(nx1=24, nx2=40, deck="straka.yaml")]
    ws = [problems.straka(o, "cpu", xc=1000.0, zc=1200.0, xr=800.0, zr=600.0)
          for o in members]
    rs = [torch.from_numpy(ratios(o)) for o in members]
    ens = Ensemble(members, device=cuda, graphs=False)
    ens.initialize(ws, autotune=False, rs=rs)
    dts = []
    for _ in range(5):
        dt = ens.max_time_step().clone()
        dts.append(dt)
        ens.step(dt)
    for k, o in enumerate(members):
        blk = sg.MeshBlock(o).to(cuda)
        vars = {"hydro_w": ws[k].to(cuda), "scalar_r": rs[k].to(cuda)}
        blk.initialize(vars)
        for dt in dts:
            blk.step(vars, float(dt[k]))
        assert torch.equal(ens.scalars(k), vars["scalar_s"]), k
        assert torch.equal(ens.state(k), vars["hydro_u"]), k


@pytest.mark.parametrize("cov", [False, True])
def test_3d_scalars_against_oracle(oracle, cuda, cov):
    """A 3-D convection block (the serving deck, its vertical implicit solve
    on the (x2, x3) columns) with a tracer: FP64 with the oracle, without
    and with the covariance row (x2 and x3 faces) and its limiter."""
    cfg = copy.deepcopy(sg.options.yaml_lite.load("snapy_gb300/decks/convection3d.yaml"))
    cfg["scalar"] = {"nvar": 1}
    cfg["dynamics"]["flux-covariance"] = cov
    opts = sg.MeshBlockOptions.from_config(cfg)
    c = opts.coord()
    c.nx1, c.nx2, c.nx3 = 16, 12, 10
    c.x1max, c.x2max, c.x3max = 16 * 50.0, 12 * 50.0, 10 * 50.0
    opts.hydro().precision = "float64"
    opts.execution = "eager"
    opts.autotune = False
    w = problems.convection3d(opts, "cpu", seed=7)
    z = np.linspace(0.0, 1.0, c.nc1)[None, None, None, :]
    r = (1e-3 * (1.0 + 0.5 * np.sin(5.0 * z))) * np.ones((1, c.nc3, c.nc2, c.nc1))
    blk = sg.MeshBlock(opts).to(cuda)
    vars = {"hydro_w": w.to(cuda), "scalar_r": torch.from_numpy(r).to(cuda)}
    blk.initialize(vars)
    ob = oracle.block_from_options(opts)
    u = ob.initialize(w.numpy())
    s = ob.set_scalars(u[0] * r)
    for _ in range(4):
        dt = blk.max_time_step(vars)
        blk.step(vars, dt)
        ob.step(u, dt)
    got = vars["scalar_s"].double().cpu().numpy()
    inner = (slice(None), slice(3, -3), slice(3, -3), slice(3, -3))
    e = rel(got[inner], s[inner])
    print(f"\n3-D tracer vs oracle: rel L2 {e:.2e}")
    assert e <= 1e-12
