"""The vertical implicit solve's failure path, as the reference's own tests
drive it (tests/test_lu_failure.cpp:177-499): a column whose block LU meets a
non-finite input fails, is marked in its solution and keeps its explicit
tendency, the block's status reports the failure (check flag bit 32), the
other columns keep their solution, the retry restores the step's input, and
the refined FP32 solve hands exactly the failed columns to the FP64 solve.

The failure is made on the host: one interior cell of the state is set to
NaN before the stage (no GPU fault is involved).  The x2 reconstruction
spreads it to the columns whose stencils read that cell (three either side),
so those columns fail, and no other.
"""
import numpy as np
import pytest
import torch

import snapy_gb300 as sg
from snapy_gb300 import problems

pytestmark = pytest.mark.gpu

STRAKA = "snapy_gb300/decks/straka.yaml"
NX1, NX2 = 48, 40
BAD_J, BAD_I = 20, 10  # the planted cell: interior column and layer
VIC_FAILED = 32        # check flag: a column of the implicit solve failed


def window(precision="float64"):
    opts = sg.MeshBlockOptions.from_yaml(STRAKA)
    c = opts.coord()
    c.nx1, c.nx2, c.x1max, c.x2max = NX1, NX2, NX1 * 50.0, NX2 * 50.0
    opts.execution = "eager"
    opts.autotune = False
    opts.hydro().precision = precision
    if precision == "float32":
        opts.hydro().icorr.precision = "float32"  # the refined solve
    return opts


def planted(opts, cuda):
    """A block on the Straka window, the dt of its clean state, and the
    state with one interior density set to NaN."""
    blk = sg.MeshBlock(opts).to(cuda)
    w = problems.straka(opts, "cpu", xc=1000.0, zc=1200.0, xr=800.0, zr=600.0)
    vars = {"hydro_w": w.to(cuda)}
    blk.initialize(vars)
    dt = blk.max_time_step(vars)
    ng = opts.coord().nghost
    vars["hydro_u"][0, 0, ng + BAD_J, ng + BAD_I] = float("nan")
    return blk, vars, w, dt


def nan_columns(u, ng):
    """Interior x2 columns (0-based) holding any NaN."""
    core = u[:, 0, ng:-ng, ng:-ng]
    return sorted(np.nonzero(np.isnan(core).any(axis=(0, 2)))[0].tolist())


def test_failed_columns_are_isolated_and_flagged(oracle, cuda):
    opts = window()
    blk, vars, w, dt = planted(opts, cuda)
    ob = oracle.block_from_options(opts)
    u = ob.initialize(w.numpy())
    ng = opts.coord().nghost
    u[0, 0, ng + BAD_J, ng + BAD_I] = np.nan
    blk.forward(vars, dt, 0)
    ob.stage(u, dt, 0)
    got = vars["hydro_u"].cpu().numpy()
    bad = nan_columns(got, ng)
    # the columns whose x2 stencils read the planted cell, and no other
    assert bad == list(range(BAD_J - 3, BAD_J + 4)), bad
    assert nan_columns(u, ng) == bad
    # every other column is the oracle's, bit for bit as in the clean runs
    good = np.ones(NX2 + 2 * ng, dtype=bool)
    good[[ng + j for j in bad]] = False
    good[:ng] = good[-ng:] = False
    a, b = got[:, 0, good, ng:-ng], u[:, 0, good, ng:-ng]
    assert np.isfinite(a).all()
    for v in range(5):
        den = np.linalg.norm(b[v])
        err = np.linalg.norm(a[v] - b[v]) / (den if den > 0 else 1.0)
        assert err <= 1e-12, (v, err)
    flags = int(blk.batch.check()[0].item())
    assert flags & VIC_FAILED, flags


def test_retry_restores_the_step(cuda):
    """check_redo after a step with failed columns: a redo (> 0) and the
    state back at the step's input (MeshBlockImpl::apply_redo)."""
    opts = window()
    blk, vars, w, dt = planted(opts, cuda)
    saved = vars["hydro_u"].clone()
    blk.step(vars, dt)
    assert blk.check_redo(vars) == 1
    a, b = vars["hydro_u"].cpu().numpy(), saved.cpu().numpy()
    assert np.array_equal(np.isnan(a), np.isnan(b))
    assert np.array_equal(a[~np.isnan(a)], b[~np.isnan(b)])


def test_a_clean_step_after_the_failure_is_accepted(cuda):
    """The status is cleared by the check: the same block, its state
    repaired, steps and is accepted (the reference's reset_status)."""
    opts = window()
    blk, vars, w, dt = planted(opts, cuda)
    blk.step(vars, dt)
    assert blk.check_redo(vars) == 1
    ng = opts.coord().nghost
    clean = sg.MeshBlock(opts).to(cuda)
    cv = {"hydro_w": w.to(cuda)}
    clean.initialize(cv)
    vars["hydro_u"][0, 0, ng + BAD_J, ng + BAD_I] = cv["hydro_u"][0, 0, ng + BAD_J,
                                                                 ng + BAD_I]
    blk.step(vars, dt)
    assert blk.check_redo(vars) == 0


def test_refined_solve_hands_the_failed_columns_to_fp64(cuda):
    """implicit-precision float32: the FP32 sweep of a failed column does
    not converge, so the refined solve masks it for the direct FP64 solve
    (counted as the reference's implicit.fp64_columns), which fails too and
    marks it; exactly the columns the planted cell reaches."""
    opts = window("float32")
    blk, vars, w, dt = planted(opts, cuda)
    assert blk.batch.solve_fallbacks()[0] == 0
    blk.forward(vars, dt, 0)
    torch.cuda.synchronize()
    ng = opts.coord().nghost
    bad = nan_columns(vars["hydro_u"].cpu().numpy(), ng)
    assert bad == list(range(BAD_J - 3, BAD_J + 4)), bad
    assert blk.batch.solve_fallbacks()[0] == len(bad)
    assert int(blk.batch.check()[0].item()) & VIC_FAILED
