"""The register monitor's counts and the budget's restart carry.

* riemann.pstar_clamp (src/riemann/riemann.cpp:330-339): a 1-D tube whose
  two halves move apart at 1.5 (c = 0.75) makes HLLC clamp its contact
  pressure at the centre; the device's count of interior faces with a
  clamped contact pressure equals the oracle's, step by step, with the
  states bitwise the oracle's.
* implicit.fp64_columns (src/hydro/hydro.cpp:460-470): the columns the
  refined FP32 solve leaves to its FP64 retry, counted in the step's
  monitor slot as in the running count.
* The budget's record carries the reference's counter and minimum names,
  and an interval open at a restart (BudgetCarry) resumes in a fresh block:
  the interrupted run's record equals the uninterrupted one's.
"""
import copy

import numpy as np
import pytest
import torch

import snapy_gb300 as sg
from snapy_gb300 import budget as Bg, problems, restart as R

pytestmark = pytest.mark.gpu


def tube(cuda, nx1=128):
    opts = sg.MeshBlockOptions.from_yaml("snapy_gb300/decks/sod.yaml")
    c = opts.coord()
    c.nx1 = nx1
    opts.execution = "eager"
    opts.autotune = False
    w = torch.zeros((5, 1, 1, c.nc1), dtype=torch.float64)
    x = torch.as_tensor(0.5 * (np.asarray(c.faces(1))[:-1] + np.asarray(c.faces(1))[1:]))
    w[0] = 1.0
    w[4] = 0.4
    w[1, 0, 0] = torch.where(x < 0.5, -1.5, 1.5)
    return opts, w


def test_hllc_clamp_counts_match_oracle(oracle, cuda):
    opts, w = tube(cuda)
    blk = sg.MeshBlock(opts).to(cuda)
    vars = {"hydro_w": w.to(cuda)}
    blk.initialize(vars)
    ob = oracle.block_from_options(opts)
    u = ob.initialize(w.numpy())
    mon = ob.count_monitor()
    acc = torch.zeros((1, 2), dtype=torch.int64, device=cuda)
    seen = []
    for _ in range(8):
        dt = blk.max_time_step(vars)
        before = int(mon[0])
        blk.step(vars, dt)
        assert blk.check_redo(vars) == 0
        ob.step(u, dt)
        acc.zero_()
        blk.batch.add_step_counts(acc)
        got = int(acc[0, 0].item())
        assert got == int(mon[0]) - before, (got, int(mon[0]) - before)
        assert np.array_equal(vars["hydro_u"].cpu().numpy(), u)
        seen.append(got)
    # the clamp happens, at the centre faces while the halves separate
    assert seen[0] > 0, seen


def test_fp64_columns_in_the_step_count(cuda):
    """A NaN planted in one interior cell of an FP32 block with the refined
    solve: the columns its stencils reach go to the FP64 retry; the step's
    monitor count and the running count both have them."""
    opts = sg.MeshBlockOptions.from_yaml("snapy_gb300/decks/straka.yaml")
    c = opts.coord()
    c.nx1, c.nx2, c.x1max, c.x2max = 48, 40, 48 * 50.0, 40 * 50.0
    opts.execution = "eager"
    opts.autotune = False
    opts.hydro().precision = "float32"
    opts.hydro().icorr.precision = "float32"
    blk = sg.MeshBlock(opts).to(cuda)
    vars = {"hydro_w": problems.straka(opts, "cpu", xc=1000.0, zc=1200.0,
                                       xr=800.0, zr=600.0).to(cuda)}
    blk.initialize(vars)
    dt = blk.max_time_step(vars)
    ng = c.nghost
    vars["hydro_u"][0, 0, ng + 20, ng + 10] = float("nan")
    f0 = blk.batch.solve_fallbacks()[0]
    blk.forward(vars, dt, 0)
    acc = torch.zeros((1, 2), dtype=torch.int64, device=cuda)
    blk.batch.add_step_counts(acc)
    n = blk.batch.solve_fallbacks()[0] - f0
    assert n == 7, n
    assert int(acc[0, 1].item()) == n
    assert int(acc[0, 0].item()) == 0  # LMARS: no contact-pressure clamp


def straka(cuda):
    cfg = copy.deepcopy(sg.options.yaml_lite.load("snapy_gb300/decks/straka.yaml"))
    opts = sg.MeshBlockOptions.from_config(cfg)
    c = opts.coord()
    c.nx1, c.nx2, c.x1max, c.x2max = 40, 48, 40 * 50.0, 48 * 50.0
    opts.autotune = False
    return opts


def start(opts, cuda):
    blk = sg.MeshBlock(opts).to(cuda)
    vars = {"hydro_w": problems.straka(opts, cuda, xc=1200.0, zc=1000.0,
                                       xr=600.0, zr=500.0)}
    blk.initialize(vars)
    con = Bg.BudgetConsumer()
    con.bind(blk)
    return blk, vars, con


def advance(blk, vars, con, n, t):
    for _ in range(n):
        dt = blk.max_time_step(vars)
        blk.step(vars, dt)
        assert blk.check_redo(vars) == 0
        blk.cycle += 1
        t += dt
        con.observe(blk, vars, dt)
    return t


def test_record_names_and_the_carry_across_a_restart(cuda, tmp_path):
    opts = straka(cuda)
    # the uninterrupted run: its first step starts the interval, 7 follow
    blk, vars, con = start(opts, cuda)
    t = advance(blk, vars, con, 8, 0.0)
    whole = con.flush(blk, vars, t)
    assert whole.counters == Bg.COUNTERS and whole.minima == Bg.MINIMA
    assert whole.counter.dtype == np.int64 and (whole.counter == 0).all()
    assert np.isinf(whole.minimum).all()
    # the interrupted run: a restart after 4 steps carries the open interval
    blk, vars, con = start(opts, cuda)
    t = advance(blk, vars, con, 4, 0.0)
    path = blk.write_restart(vars, str(tmp_path), "carry", number=1, time=t,
                             budget=con)
    data = R.load_restart(path)
    assert Bg.CARRY_PREFIX + "total_prev" in data
    again = sg.MeshBlock(opts).to(cuda)
    vars2 = {"hydro_w": problems.straka(opts, cuda, xc=1200.0, zc=1000.0,
                                        xr=600.0, zr=500.0)}
    again.initialize(vars2)
    con2 = Bg.BudgetConsumer()
    con2.bind(again)
    t2 = again.initialize_from_restart(vars2, path, budget=con2)
    assert t2 == t
    t2 = advance(again, vars2, con2, 4, t2)
    part = con2.flush(again, vars2, t2)
    assert part.interval == whole.interval
    for k in ("total", "change", "boundary", "counter"):
        assert np.array_equal(getattr(part, k), getattr(whole, k)), k
    # a carry read back is not state: the next restart writes its own only
    p2 = again.write_restart(vars2, str(tmp_path), "carry", number=2, time=t2)
    assert not any(k.startswith(Bg.CARRY_PREFIX) for k in R.load_restart(p2))
