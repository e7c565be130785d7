"""The partial matrix of the vertical implicit solve (implicit-scheme 1: the
3x3 blocks of rows and columns {rho, m1, E}, the tangential momenta folded
into the density column and carried by the face mass transfers) on the GPU
against the oracle's restatement (src/implicit/vic_assemble_impl.h:152-214,
forward_sweep_impl.h:30-131, vic_redistribute_impl.h:178-200,
implicit_hydro.cpp:520-530,662-666).

FP64 within 1e-12 relative L2 per field of the oracle: Straka windows (the
warp-form finish; the thread form on a batch of 20,480 columns; x2 cells 40
times the x1 ones, vertical acoustic Courant number near 40), the x1 step
field with the partial matrix's momentum posts, a 3-D convection block, a
tracer; FP32 state within 1e-5 of the FP64 oracle, with the blocks assembled
in FP64 or in FP32; a resting column stays at rest; members of both schemes
in one batch each equal the member alone."""
import copy

import numpy as np
import pytest
import torch

import snapy_gb300 as sg
from snapy_gb300 import problems
from snapy_gb300.ensemble import Ensemble

pytestmark = pytest.mark.gpu

TOL = 1e-12


def rel_l2(a, b):
    out = []
    for v in range(a.shape[0]):
        den = np.linalg.norm(b[v])
        num = np.linalg.norm(a[v] - b[v])
        out.append(num / den if den > 0 else num)
    return np.array(out)


def straka(scheme=1, nx1=48, nx2=40, dx2=50.0, precision="float64", tracer=False):
    cfg = copy.deepcopy(sg.options.yaml_lite.load("snapy_gb300/decks/straka.yaml"))
    cfg["integration"]["implicit-scheme"] = scheme
    if tracer:
        cfg["scalar"] = {"nvar": 1}
    opts = sg.MeshBlockOptions.from_config(cfg)
    c = opts.coord()
    c.nx1, c.nx2, c.x1max, c.x2max = nx1, nx2, nx1 * 50.0, nx2 * dx2
    opts.hydro().precision = precision
    opts.execution = "eager"
    return opts


def bubble(opts, xc=1000.0, zc=1200.0, xr=800.0, zr=600.0):
    return problems.straka(opts, "cpu", xc=xc, zc=zc, xr=xr, zr=zr)


def run_pair(oracle, cuda, opts, w, nsteps, check=True, scalar_r=None):
    blk = sg.MeshBlock(opts).to(cuda)
    vars = {"hydro_w": w.to(cuda)}
    if scalar_r is not None:
        vars["scalar_r"] = torch.from_numpy(scalar_r).to(cuda)
    blk.initialize(vars)
    ob = oracle.block_from_options(opts)
    u = ob.initialize(w.numpy())
    s = ob.set_scalars(u[0] * scalar_r) if scalar_r is not None else None
    errs = []
    for _ in range(nsteps):
        dt = blk.max_time_step(vars)
        blk.step(vars, dt)
        assert blk.check_redo(vars) == 0
        ob.step(u, dt)
        if check:
            errs.append(rel_l2(blk.total_u(vars).double().cpu().numpy(), u).max())
    return blk, vars, u, s, errs


@pytest.mark.parametrize("dx2", [50.0, 2000.0])
def test_fp64_parity(oracle, cuda, dx2):
    opts = straka(dx2=dx2)
    w = bubble(opts, xc=0.5 * opts.coord().x2max, xr=0.3 * opts.coord().x2max)
    _, _, _, _, errs = run_pair(oracle, cuda, opts, w, 6)
    print(f"\nscheme 1, dx2 {dx2}: max rel L2 per step {['%.1e' % e for e in errs]}")
    assert max(errs) <= TOL


def test_fp64_parity_wide_batch(oracle, cuda):
    """20,480 columns: the thread-per-column finish."""
    opts = straka(nx1=6, nx2=20480)
    w = problems.straka(opts, "cpu", xc=5000.0, zc=150.0, xr=2000.0, zr=100.0)
    _, _, _, _, errs = run_pair(oracle, cuda, opts, w, 2)
    assert max(errs) <= TOL


def test_step_field_posts(oracle, cuda):
    """S_1 carries the partial matrix's posts: the dry transfer on row IDN
    and the donor transfer q w_t on rows IVY and IVZ."""
    opts = straka()
    w = bubble(opts)
    blk = sg.MeshBlock(opts).to(cuda)
    reg = blk.flux_register()
    reg.request_step_field(1)
    vars = {"hydro_w": w.to(cuda)}
    blk.initialize(vars)
    ob = oracle.block_from_options(opts)
    u = ob.initialize(w.numpy())
    S1 = ob.request_step_field(1)
    for _ in range(3):
        dt = blk.max_time_step(vars)
        for s in range(3):
            blk.forward(vars, dt, s)
            ob.stage(u, dt, s)
        assert blk.check_redo(vars) == 0
        err = rel_l2(reg.step_field(1).cpu().numpy(), S1)
        assert err.max() <= TOL, err
    assert np.abs(S1[2]).max() > 0  # the IVY row holds the transfers


def test_3d_block(oracle, cuda):
    cfg = copy.deepcopy(sg.options.yaml_lite.load("snapy_gb300/decks/convection3d.yaml"))
    cfg["integration"]["implicit-scheme"] = 1
    opts = sg.MeshBlockOptions.from_config(cfg)
    c = opts.coord()
    c.nx1, c.nx2, c.nx3 = 16, 12, 10
    c.x1max, c.x2max, c.x3max = 16 * 50.0, 12 * 50.0, 10 * 50.0
    opts.hydro().precision = "float64"
    opts.execution = "eager"
    w = problems.convection3d(opts, "cpu", seed=7)
    _, _, _, _, errs = run_pair(oracle, cuda, opts, w, 4)
    print(f"\n3-D scheme 1: max rel L2 {max(errs):.1e}")
    assert max(errs) <= TOL


def test_tracer(oracle, cuda):
    opts = straka(tracer=True)
    w = bubble(opts)
    c = opts.coord()
    z = np.linspace(0.0, 1.0, c.nc1)[None, None, None, :]
    r = (1e-3 * (1.0 + 0.5 * np.sin(5.0 * z))) * np.ones((1, c.nc3, c.nc2, c.nc1))
    _, vars, _, s, errs = run_pair(oracle, cuda, opts, w, 5, scalar_r=r)
    got = vars["scalar_s"].double().cpu().numpy()
    inner = (slice(None), slice(None), slice(3, -3), slice(3, -3))
    e = rel_l2(got[inner], s[inner]).max()
    assert max(errs) <= TOL and e <= TOL, (errs, e)


def test_fp32_state(oracle, cuda):
    """FP32 anomalies about the FP64 base, the partial blocks assembled in
    FP64: within 1e-5 of the FP64 oracle after 10 steps."""
    opts = straka(precision="float32")
    w = bubble(opts)
    blk, vars, u, _, _ = run_pair(oracle, cuda, opts, w, 10, check=False)
    got = blk.total_u(vars).double().cpu().numpy()
    inner = (slice(None), slice(None), slice(3, -3), slice(3, -3))
    err = rel_l2(got[inner], u[inner])
    print(f"\nFP32 scheme 1 vs FP64 oracle: {err}")
    assert err.max() <= 1e-5


def test_fp32_assembly(oracle, cuda):
    """implicit-precision float32: the partial blocks assembled in FP32 from
    the FP32 state, solved in FP64 by the 3x3 column solve (the refined
    solve is scheme 9's): within 1e-5 of the FP64 oracle after 10 steps, and
    a batch with a scheme-9 FP32 member (its refined solve beside it) gives
    each member its own result bit for bit."""
    opts = straka(precision="float32")
    opts.hydro().icorr.precision = "float32"
    w = bubble(opts)
    blk, vars, u, _, _ = run_pair(oracle, cuda, opts, w, 10, check=False)
    got = blk.total_u(vars).double().cpu().numpy()
    inner = (slice(None), slice(None), slice(3, -3), slice(3, -3))
    err = rel_l2(got[inner], u[inner])
    print(f"\nFP32 scheme 1, FP32 assembly, vs FP64 oracle: {err}")
    assert err.max() <= 1e-5
    # in one batch with a scheme-9 member whose blocks are FP32 too
    o9 = straka(scheme=9, precision="float32", nx2=24)
    o9.hydro().icorr.precision = "float32"
    o1 = straka(scheme=1, precision="float32", nx2=40)
    o1.hydro().icorr.precision = "float32"
    for o in (o9, o1):
        o.autotune = False
    ws = [bubble(o9, xc=600.0), bubble(o1)]
    alone = []
    for o, w0 in zip((o9, o1), ws):
        b = sg.MeshBlock(o).to(cuda)
        v = {"hydro_w": w0.to(cuda)}
        b.initialize(v)
        for _ in range(3):
            b.step(v, b.max_time_step(v))
            assert b.check_redo(v) == 0
        alone.append(v["hydro_u"].cpu().numpy())
    ens = Ensemble([o9, o1], cuda, graphs=False)
    ens.initialize([w0.to(cuda) for w0 in ws], autotune=False)
    for _ in range(3):
        ens.step()
    for k in range(2):
        assert np.array_equal(ens.state(k).cpu().numpy(), alone[k]), k


def test_rest_state_stays_at_rest(cuda):
    opts = straka(nx1=48, nx2=8, dx2=2000.0)
    blk = sg.MeshBlock(opts).to(cuda)
    vars = {"hydro_w": problems.straka(opts, cuda, dT=0.0)}
    blk.initialize(vars)
    for _ in range(10):
        blk.step(vars, blk.max_time_step(vars))
    assert blk.prim()[1:4].abs().max().item() < 1e-9


def test_both_schemes_in_one_batch(cuda):
    """A batch holding members of both schemes runs both column solves; each
    member equals itself alone, bit for bit."""
    members = problems.ensemble_members(n=2, seed=5, deck="straka.yaml",
                                        nx2_choices=(24, 40), nx1_choices=(32,))
    (o0, w0), (o1, w1) = members
    o1 = copy.deepcopy(o1)
    o1.hydro().icorr.scheme = 1
    pairs = [(o0, w0), (o1, w1)]
    ens = Ensemble([o for o, _ in pairs], device=cuda, graphs=False)
    ens.initialize([w for _, w in pairs], autotune=False)
    dts = []
    for _ in range(4):
        dt = ens.max_time_step().clone()
        dts.append(dt)
        ens.step(dt)
    for k, (o, w) in enumerate(pairs):
        blk = sg.MeshBlock(o).to(cuda)
        vars = {"hydro_w": w.to(cuda)}
        blk.initialize(vars)
        for dt in dts:
            blk.step(vars, float(dt[k]))
        assert torch.equal(ens.state(k), vars["hydro_u"]), k
