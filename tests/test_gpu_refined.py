"""The refined implicit solve of implicit-precision float32 blocks (FP32
block-Thomas sweeps corrected with FP64 residuals) against the direct FP64
solve of the same FP32-assembled system (sg_set_solve(h, 0)): the solution
of every column to FP64 roundoff with one, two and three corrections, few
columns left to the direct solve (the implicit.fp64_columns count), and the
whole FP32 run within the FP32 bar of the FP64 oracle."""
import numpy as np
import pytest
import torch

import snapy_gb300 as sg
from snapy_gb300 import _lib, problems

pytestmark = pytest.mark.gpu


def straka_fp32(nx1=48, nx2=40):
    opts = sg.MeshBlockOptions.from_yaml("snapy_gb300/decks/straka.yaml")
    c = opts.coord()
    c.nx1, c.nx2, c.x1max, c.x2max = nx1, nx2, nx1 * 50.0, nx2 * 50.0
    opts.hydro().precision = "float32"
    opts.hydro().icorr.precision = "float32"
    opts.execution = "eager"
    opts.autotune = False
    return opts


def one_stage(cuda, opts, w, corrections):
    """One stage; the solution D (du / dt_corr after the Woodbury step) of
    every column, and the columns the refined solve left to FP64."""
    blk = sg.MeshBlock(opts).to(cuda)
    vars = {"hydro_w": w.to(cuda)}
    blk.initialize(vars)
    L = _lib.load()
    blk.batch.set_solve(corrections)
    dt = blk.max_time_step(vars)
    blk.forward(vars, dt, 0)
    torch.cuda.synchronize()
    c = opts.coord()
    cells = c.nx1 * c.nx2
    D = blk.batch.scratch[0][85 * cells:90 * cells].clone()
    return D, blk.batch.solve_fallbacks()[0]


@pytest.mark.parametrize("corrections", [1, 2, 3])
def test_refined_solution_is_the_direct_one(cuda, corrections):
    opts = straka_fp32()
    w = problems.straka(opts, "cpu", xc=1000.0, zc=1200.0, xr=800.0, zr=600.0)
    Dr, fellback = one_stage(cuda, opts, w, corrections)
    Dd, none = one_stage(cuda, opts, w, 0)
    rel = (torch.linalg.norm(Dr - Dd) / torch.linalg.norm(Dd)).item()
    ncol = opts.coord().nx2
    print(f"\n{corrections} corrections vs the direct FP64 solve: rel L2 "
          f"{rel:.2e}, {fellback} of {ncol} columns left to the direct solve")
    assert none == 0
    assert 0 <= fellback <= ncol
    assert rel <= 1e-13
    if corrections >= 2:
        assert fellback <= ncol // 20


def test_refined_run_against_fp64_oracle(oracle, cuda):
    opts = straka_fp32()
    w = problems.straka(opts, "cpu", xc=1000.0, zc=1200.0, xr=800.0, zr=600.0)
    blk = sg.MeshBlock(opts).to(cuda)
    vars = {"hydro_w": w.to(cuda)}
    blk.initialize(vars)
    ob = oracle.block_from_options(opts)
    u = ob.initialize(w.numpy())
    for _ in range(10):
        dt = blk.max_time_step(vars)
        blk.step(vars, dt)
        assert blk.check_redo(vars) == 0
        ob.step(u, dt)
    got = blk.total_u(vars).double().cpu().numpy()
    err = [np.linalg.norm(got[v] - u[v]) / max(np.linalg.norm(u[v]), 1e-300)
           for v in range(5)]
    print("\nFP32 + refined solve vs FP64 oracle, rel L2 per field:",
          np.array2string(np.array(err), precision=2))
    assert max(err) <= 1e-5
    assert blk.batch.solve_fallbacks()[0] <= 10 * 3 * opts.coord().nx2 // 20


def test_refined_solution_on_3d_columns(cuda):
    """A 3-D convection block (the serving deck: FP32 state, implicit-precision
    float32, the solve on the (x2, x3) columns): the refined solution equals
    the direct FP64 one to FP64 roundoff, with few columns left to it."""
    opts = sg.MeshBlockOptions.from_yaml("snapy_gb300/decks/convection3d.yaml")
    c = opts.coord()
    c.nx1, c.nx2, c.nx3 = 24, 12, 10
    c.x1max, c.x2max, c.x3max = 24 * 50.0, 12 * 50.0, 10 * 50.0
    opts.hydro().precision = "float32"
    opts.hydro().icorr.precision = "float32"
    opts.execution = "eager"
    opts.autotune = False
    w = problems.convection3d(opts, "cpu", seed=11)
    cells = c.nx1 * c.nx2 * c.nx3
    out = []
    for k in (2, 0):
        blk = sg.MeshBlock(opts).to(cuda)
        vars = {"hydro_w": w.to(cuda)}
        blk.initialize(vars)
        blk.batch.set_solve(k)
        dt = blk.max_time_step(vars)
        blk.forward(vars, dt, 0)
        torch.cuda.synchronize()
        out.append((blk.batch.scratch[0][85 * cells:90 * cells].clone(),
                    blk.batch.solve_fallbacks()[0]))
    (Dr, fell), (Dd, none) = out
    rel = (torch.linalg.norm(Dr - Dd) / torch.linalg.norm(Dd)).item()
    ncol = c.nx2 * c.nx3
    print(f"\n3-D refined vs direct FP64 solve: rel L2 {rel:.2e}, {fell} of "
          f"{ncol} columns left to the direct solve")
    assert none == 0 and 0 <= fell <= ncol // 20
    assert rel <= 1e-13


def test_fp32_solve_against_direct_and_oracle(oracle, cuda):
    """implicit-solve fp32 (sg_set_solve(h, -1)), the reference's own FP32
    compute of the implicit solve: the FP32 sweep and its Woodbury step with
    no corrections.  Its solution is within FP32 roundoff times the
    column's condition (1.2e-5 here) of the direct FP64 one, no column fails
    on this block, and a 10-step run stays within 1e-4 of the FP64 oracle
    (2.8e-5 measured: this form is not held to the 1e-5 bar of the refined
    and direct forms)."""
    opts = straka_fp32()
    w = problems.straka(opts, "cpu", xc=1000.0, zc=1200.0, xr=800.0, zr=600.0)
    Df, fell = one_stage(cuda, opts, w, -1)
    Dd, _ = one_stage(cuda, opts, w, 0)
    rel = (torch.linalg.norm(Df - Dd) / torch.linalg.norm(Dd)).item()
    print(f"\nFP32 solve vs the direct FP64 solve: rel L2 {rel:.2e}, "
          f"{fell} columns left to the direct solve")
    assert rel <= 1e-4 and fell == 0
    opts.implicit_solve = "fp32"
    assert opts.solve_corrections() == -1
    blk = sg.MeshBlock(opts).to(cuda)
    vars = {"hydro_w": w.to(cuda)}
    blk.initialize(vars)
    ob = oracle.block_from_options(opts)
    u = ob.initialize(w.numpy())
    for _ in range(10):
        dt = blk.max_time_step(vars)
        blk.step(vars, dt)
        assert blk.check_redo(vars) == 0
        ob.step(u, dt)
    got = blk.total_u(vars).double().cpu().numpy()
    err = [np.linalg.norm(got[v] - u[v]) / max(np.linalg.norm(u[v]), 1e-300)
           for v in range(5)]
    print("FP32 state + FP32 solve vs FP64 oracle, rel L2 per field:",
          np.array2string(np.array(err), precision=2))
    assert max(err) <= 1e-4
