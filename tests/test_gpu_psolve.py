"""The partitioned (layer-parallel) form of the scheme-9 column solve
(integration/implicit-sweep: partitioned): each column cut into four chunks
swept at once by one warp, a 3-row system of the separator layers, every
layer from the separators, the Woodbury step of the wall rows.  Its
elimination order differs from the reference's serial sweep
(src/implicit/forward_sweep_impl.h:30-131), so it is held to the parity
bar, relative L2 1e-12 per field against the CPU oracle, not bit for bit:

* Straka windows whose layer counts leave every chunk remainder (16 to 65
  layers), the full 512 x 128 Straka block (3 steps, mass to round-off),
  a 3-D convection block, and an ensemble mixing short (serial) and long
  (partitioned) columns.  Each field is within 1e-12 of the oracle, or, for
  a field the oracle itself moves by more than 1e-13 when its input state
  is perturbed by one ulp, within 10 times that move.  Near rest the
  horizontal momentum is such a field: it starts at zero and grows from
  horizontal differences of the pressure, so after a step it is small
  against the rounding of the 1e5 Pa pressure around it, and any other
  order of elimination than the reference's own moves it by about 1e-9 of
  its norm.  The solution of every column, the solve's own output, is
  within 1e-12 (normwise, per block) of the serial solve's, which is the
  oracle's bit for bit;
* the failure path: a column the partitioned form cannot solve goes back to
  the serial solve, which fails it exactly as the reference does (the same
  columns marked, the same flag) and counts it;
* columns shorter than 16 layers and scheme-1 blocks keep their own solve,
  bit for bit;
* the form's reciprocal (two Newton-Raphson steps from an FP32 seed) is
  within one ulp of the IEEE division;
* the autotuner's choice (implicit-sweep: auto) is recorded and gives the
  same solution to rounding.
"""
import numpy as np
import pytest
import torch

import snapy_gb300 as sg
from snapy_gb300 import _lib, problems
from snapy_gb300.ensemble import Ensemble

pytestmark = pytest.mark.gpu

TOL = 1e-12
STRAKA = "snapy_gb300/decks/straka.yaml"
VIC_FAILED = 32


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    out = []
    for v in range(a.shape[0]):
        den = np.linalg.norm(b[v])
        num = np.linalg.norm(a[v] - b[v])
        out.append(num / den if den > 0 else num)
    return np.array(out)


def window(nx1, nx2, sweep="partitioned", scheme=9):
    opts = sg.MeshBlockOptions.from_yaml(STRAKA)
    c = opts.coord()
    c.nx1, c.nx2, c.x1max, c.x2max = nx1, nx2, nx1 * 50.0, nx2 * 50.0
    opts.execution = "eager"
    opts.autotune = False
    opts.implicit_sweep = sweep
    opts.hydro().icorr.scheme = scheme
    return opts


def bubble(opts):
    c = opts.coord()
    return problems.straka(opts, "cpu", xc=0.4 * c.x2max, zc=0.45 * c.x1max,
                           xr=0.2 * c.x2max, zr=0.25 * c.x1max)


def ulp_floor(oracle, opts, w, dts, seed=3):
    """Per step and field, how far the oracle's own state moves over the
    steps of dts when its initial conserved state is perturbed by one ulp (a
    random sign per interior cell and variable): the rounding sensitivity
    of the reference's path at this state."""
    ob = oracle.block_from_options(opts)
    u = ob.initialize(w.numpy())
    v = u.copy()
    rng = np.random.default_rng(seed)
    sign = rng.choice([-1.0, 1.0], size=v.shape)
    pert = np.nextafter(v, v + sign * np.abs(v) + sign)
    c = opts.coord()
    ng = c.nghost
    core = [slice(None)] + [slice(ng, -ng) if nc > 1 else slice(None)
                            for nc in (c.nc3, c.nc2, c.nc1)]
    v[tuple(core)] = pert[tuple(core)]
    out = []
    for dt in dts:
        for s in range(3):
            ob.stage(u, dt, s)
            ob.stage(v, dt, s)
        out.append(rel_l2(v, u))
    return out


def bar(floor):
    """The per-field tolerance of a non-bitwise elimination order."""
    return np.maximum(TOL, np.where(floor > 1e-13, 10.0 * floor, TOL))


def run_pair(oracle, cuda, opts, w, steps=3):
    """The GPU block and the oracle over `steps` RK3 steps at the GPU's dt;
    returns the GPU block, its state, the per-field relative L2 after each
    step and the oracle's one-ulp floor over the same steps."""
    blk = sg.MeshBlock(opts).to(cuda)
    vars = {"hydro_w": w.to(cuda)}
    blk.initialize(vars)
    ob = oracle.block_from_options(opts)
    u = ob.initialize(w.numpy())
    errs, dts = [], []
    for _ in range(steps):
        dt = blk.max_time_step(vars)
        dts.append(dt)
        for s in range(3):
            blk.forward(vars, dt, s)
            ob.stage(u, dt, s)
        assert blk.check_redo(vars) == 0
        errs.append(rel_l2(vars["hydro_u"].cpu().numpy(), u))
    return blk, vars, u, errs, ulp_floor(oracle, opts, w, dts)


def within(errs, floors):
    """Every step's per-field error within the bar of that step's floor."""
    ok = all((e <= bar(f)).all() for e, f in zip(errs, floors))
    return ok, list(zip(errs, floors))


@pytest.mark.parametrize("nx1", [16, 19, 48, 65])
def test_partitioned_window_parity(oracle, cuda, nx1):
    opts = window(nx1, 40)
    blk, vars, u, errs, floor = run_pair(oracle, cuda, opts, bubble(opts))
    assert blk.batch.sweep() == 1
    ok, info = within(errs, floor)
    assert ok, info
    # no column needed the serial solve
    assert blk.batch.solve_fallbacks()[0] == 0


def test_partitioned_straka_512x128_parity(oracle, cuda):
    opts = sg.MeshBlockOptions.from_yaml(STRAKA)
    opts.execution = "eager"
    opts.implicit_sweep = "partitioned"
    w = problems.straka(opts, "cpu")
    blk, vars, u, errs, floor = run_pair(oracle, cuda, opts, w)
    assert blk.batch.sweep() == 1
    ok, info = within(errs, floor)
    assert ok, info
    c = opts.coord()
    ng = c.nghost
    got = vars["hydro_u"].cpu().numpy()
    w0 = problems.straka(opts, "cpu").numpy()
    ob = oracle.block_from_options(opts)
    m0 = ob.initialize(w0)[0, 0, ng:ng + c.nx2, ng:ng + c.nx1].sum()
    m1 = got[0, 0, ng:ng + c.nx2, ng:ng + c.nx1].sum()
    assert abs(m1 - m0) <= 1e-13 * m0
    assert blk.batch.solve_fallbacks()[0] == 0


def test_partitioned_3d_parity(oracle, cuda):
    opts = sg.MeshBlockOptions.from_yaml("snapy_gb300/decks/convection3d.yaml")
    c = opts.coord()
    c.nx1, c.nx2, c.nx3 = 24, 12, 10
    c.x1max, c.x2max, c.x3max = 24 * 50.0, 12 * 50.0, 10 * 50.0
    opts.hydro().precision = "float64"
    opts.problem["dtheta"] = 2.0
    opts.problem["layer"] = 0.4
    opts.execution = "eager"
    opts.autotune = False
    opts.implicit_sweep = "partitioned"
    w = problems.convection3d(opts, "cpu", seed=11)
    blk, vars, u, errs, floor = run_pair(oracle, cuda, opts, w)
    assert blk.batch.sweep() == 1
    ok, info = within(errs, floor)
    assert ok, info


@pytest.mark.parametrize("shape", [(48, 40), (128, 512)])
def test_solution_is_the_serial_one_to_rounding(cuda, shape):
    """The solve's own output, the solution D of every column after the
    Woodbury step (the finish reads it and leaves it), of one stage from
    the same state: normwise within 1e-12 of the serial solve's."""
    nx1, nx2 = shape
    Ds = []
    for sweep in ("serial", "partitioned"):
        opts = window(nx1, nx2, sweep)
        blk = sg.MeshBlock(opts).to(cuda)
        vars = {"hydro_w": bubble(opts).to(cuda)}
        blk.initialize(vars)
        blk.forward(vars, blk.max_time_step(vars), 0)
        torch.cuda.synchronize()
        cells = nx1 * nx2
        Ds.append(blk.batch.scratch[0][85 * cells:90 * cells].double().cpu().numpy())
    rel = np.linalg.norm(Ds[1] - Ds[0]) / np.linalg.norm(Ds[0])
    assert rel <= TOL, rel


def test_short_columns_and_scheme_1_keep_their_solve(cuda):
    """Columns under 16 layers and scheme-1 blocks: the partitioned setting
    leaves their solve alone, bit for bit."""
    for nx1, scheme in ((12, 9), (48, 1)):
        outs = []
        for sweep in ("serial", "partitioned"):
            opts = window(nx1, 24, sweep, scheme)
            blk = sg.MeshBlock(opts).to(cuda)
            vars = {"hydro_w": bubble(opts).to(cuda)}
            blk.initialize(vars)
            for _ in range(2):
                blk.step(vars, blk.max_time_step(vars))
                assert blk.check_redo(vars) == 0
            outs.append(vars["hydro_u"].cpu().numpy())
        assert np.array_equal(outs[0], outs[1]), (nx1, scheme)


def test_partitioned_ensemble_mixed_lengths(oracle, cuda):
    """One handle with members of 12 to 64 layers: the short ones take the
    serial solve, the others the partitioned one; each member against its
    own oracle block."""
    members = []
    for nx1, nx2 in ((12, 24), (40, 32), (64, 16), (33, 48)):
        members.append(window(nx1, nx2))
    ens = Ensemble(members, cuda)
    ws = [bubble(m) for m in members]
    ens.initialize([w.to(cuda) for w in ws], autotune=False)
    assert ens.batch.sweep() == 1
    obs = [oracle.block_from_options(m) for m in members]
    us = [ob.initialize(w.numpy()) for ob, w in zip(obs, ws)]
    hist = [[] for _ in members]
    for _ in range(2):
        dts = ens.max_time_step().clone()
        ens.step(dts)
        for k, (ob, u, dt) in enumerate(zip(obs, us, dts.cpu().numpy())):
            hist[k].append(float(dt))
            for s in range(3):
                ob.stage(u, float(dt), s)
    for b, u in enumerate(us):
        err = rel_l2(ens.batch.current(b).cpu().numpy(), u)
        ok, info = within([err], ulp_floor(oracle, members[b], ws[b], hist[b])[-1:])
        assert ok, (b, info)


def test_failed_columns_go_back_to_the_serial_solve(oracle, cuda):
    """A NaN planted in one interior cell: the partitioned form cannot solve
    the columns its x2 stencils reach, hands them to the serial solve,
    which fails and marks them as the reference does; the other columns
    match the oracle."""
    nx1, nx2, bj, bi = 48, 40, 20, 10
    opts = window(nx1, nx2)
    blk = sg.MeshBlock(opts).to(cuda)
    w = bubble(opts)
    vars = {"hydro_w": w.to(cuda)}
    blk.initialize(vars)
    dt = blk.max_time_step(vars)
    ng = opts.coord().nghost
    vars["hydro_u"][0, 0, ng + bj, ng + bi] = float("nan")
    ob = oracle.block_from_options(opts)
    u = ob.initialize(w.numpy())
    u[0, 0, ng + bj, ng + bi] = np.nan
    blk.forward(vars, dt, 0)
    ob.stage(u, dt, 0)
    got = vars["hydro_u"].cpu().numpy()
    core = got[:, 0, ng:-ng, ng:-ng]
    bad = sorted(np.nonzero(np.isnan(core).any(axis=(0, 2)))[0].tolist())
    assert bad == list(range(bj - 3, bj + 4)), bad
    assert blk.batch.solve_fallbacks()[0] == len(bad)
    assert int(blk.batch.check()[0].item()) & VIC_FAILED
    good = np.ones(nx2 + 2 * ng, dtype=bool)
    good[[ng + j for j in bad]] = False
    good[:ng] = good[-ng:] = False
    err = rel_l2(got[:, 0, good, ng:-ng], u[:, 0, good, ng:-ng])
    floor = ulp_floor(oracle, opts, w, [dt])[0]
    assert (err <= np.maximum(bar(floor), 1e-11)).all(), (err, floor)


def test_reciprocal_within_an_ulp(cuda):
    g = torch.Generator(device="cpu").manual_seed(5)
    m = 1.0 + torch.rand(1 << 20, generator=g, dtype=torch.float64)
    e = torch.randint(-1000, 1000, (1 << 20,), generator=g).to(torch.float64)
    s = torch.where(torch.rand(1 << 20, generator=g) < 0.5, -1.0, 1.0).double()
    x = (s * m * torch.pow(2.0, e)).to(cuda)
    # special and boundary values take the division
    x = torch.cat([x, torch.tensor([0.0, -0.0, float("inf"), 5e-324, 1e-310,
                                    1.7e308, 2.2250738585072014e-308, 1.0, -3.0],
                                   dtype=torch.float64, device=cuda)])
    r = torch.empty_like(x)
    L = _lib.load()
    _lib.check(L.sg_psw_rcp(x.data_ptr(), r.data_ptr(), x.numel(),
                            torch.cuda.current_stream().cuda_stream), "sg_psw_rcp")
    ref = 1.0 / x
    torch.cuda.synchronize()
    fin = torch.isfinite(ref) & (ref != 0)
    ulp = torch.abs(torch.nextafter(ref[fin], ref[fin] * 2) - ref[fin])
    assert (torch.abs(r[fin] - ref[fin]) <= ulp).all()
    assert torch.equal(r[~fin], ref[~fin])


def test_autotuned_sweep_is_recorded(oracle, cuda, tmp_path, monkeypatch):
    """implicit-sweep: auto: the autotuner times both forms, records its
    choice, and the solution is the serial one to rounding."""
    monkeypatch.setenv("SNAPY_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    opts = window(64, 128, "auto")
    opts.autotune = True
    blk, vars, u, errs, floor = run_pair(oracle, cuda, opts, bubble(opts), steps=2)
    sched = blk.batch.schedule
    assert sched["sweep"] in (0, 1)
    assert blk.batch.sweep() == sched["sweep"]
    ok, info = within(errs, floor)
    assert ok, info
    # a second block of the same configuration recalls it
    again = sg.MeshBlock(opts).to(cuda)
    again.initialize({"hydro_w": bubble(opts).to(cuda)})
    assert again.batch.schedule["cached"]
    assert again.batch.sweep() == sched["sweep"]
