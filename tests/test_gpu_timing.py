"""Per-kernel device timing of a stage (sg_set_timing / sg_kernel_times)."""
import os

import pytest
import torch

import snapy_gb300 as sg
from snapy_gb300 import problems

pytestmark = pytest.mark.gpu

STRAKA_VIC = os.path.join(os.path.dirname(sg.__file__), "decks", "straka.yaml")


def test_kernel_times_cover_eager_stages_only(cuda):
    opts = sg.MeshBlockOptions.from_yaml(STRAKA_VIC)
    c = opts.coord()
    c.nx1, c.nx2 = 32, 24
    c.x1max, c.x2max = 32 * 50.0, 24 * 50.0
    blk = sg.MeshBlock(opts).to(cuda)
    vars = {"hydro_w": problems.straka(opts, cuda, xc=600.0, zc=800.0,
                                       xr=300.0, zr=300.0)}
    blk.initialize(vars)
    dt = blk.max_time_step(vars)
    b = blk.batch
    # graphs of both steady buffer rotations, then replays with timing on:
    # a captured launch records no event
    for _ in range(6):
        blk.step(vars, dt)
    b.set_timing(True)
    for _ in range(2):
        blk.step(vars, dt)
    torch.cuda.synchronize()
    assert blk.execution_report()["replays"] >= 3
    assert b.kernel_times() == {}
    # eager stages: one interval per kernel and stage
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record()
    for s in range(3):
        b.stage(s)
    t1.record()
    kt = b.kernel_times()
    names = {"stage_kernel", "vic_assemble_kernel", "vic_solve_kernel",
             "vic_finish_kernel", "ghost_kernel"}
    assert set(kt) == names
    assert all(n == 3 and ms > 0 for ms, n in kt.values())
    total = sum(ms for ms, _ in kt.values())
    assert total <= t0.elapsed_time(t1) * 1.05 + 0.05
    assert b.kernel_times() == {}  # drained
    b.set_timing(False)
    b.stage(0)
    assert b.kernel_times() == {}
