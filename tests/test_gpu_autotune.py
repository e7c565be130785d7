"""The schedule autotuner: its trial launches leave the block as they found
it, the schedule it picks changes no result (bitwise), and a second handle
of the same configuration takes the choice from the cache."""
import ctypes

import pytest
import torch

import snapy_gb300 as sg
from snapy_gb300 import _lib, problems

pytestmark = pytest.mark.gpu


def straka_vic(nx1=48, nx2=40, autotune=False):
    opts = sg.MeshBlockOptions.from_yaml("snapy_gb300/decks/straka.yaml")
    c = opts.coord()
    c.nx1, c.nx2 = nx1, nx2
    c.x1max, c.x2max = nx1 * 50.0, nx2 * 50.0
    opts.autotune = autotune
    return opts


def run(cuda, opts, steps=3, before_steps=None):
    blk = sg.MeshBlock(opts).to(cuda)
    blk.flux_register().request_step_field(1)
    blk.flux_register().request_step_field(2)
    w = problems.straka(opts, "cpu", xc=1000.0, zc=1200.0, xr=800.0, zr=600.0)
    vars = {"hydro_w": w.to(cuda)}
    blk.initialize(vars)
    if before_steps:
        before_steps(blk, vars)
    for _ in range(steps):
        blk.step(vars, blk.max_time_step(vars))
        assert blk.check_redo(vars) == 0
    return blk, vars


def test_trials_leave_the_block_alone(cuda, monkeypatch, tmp_path):
    monkeypatch.setenv("SNAPY_GB300_TUNE_CACHE", "off")
    seen = {}

    def tune(blk, vars):
        b = blk.batch
        seen["u"] = vars["hydro_u"].clone()
        seen["rot"] = b.rotation()
        seen["s1"] = b.step_field(0, 1).clone()
        sch = b.autotune()
        seen["sch"] = sch
        assert b.rotation() == seen["rot"]
        assert torch.equal(vars["hydro_u"], seen["u"])
        assert torch.equal(b.step_field(0, 1), seen["s1"])
        assert int(b.check()[0].item()) == 0

    tuned, tv = run(cuda, straka_vic(), before_steps=tune)
    plain, pv = run(cuda, straka_vic())
    assert not seen["sch"]["cached"] and seen["sch"]["finish"] in (1, 2)
    assert seen["sch"]["stage_ms"] > 0 and seen["sch"]["solve_ms"] > 0
    assert torch.equal(tv["hydro_u"], pv["hydro_u"])
    for d in (1, 2):
        assert torch.equal(tuned.flux_register().step_field(d),
                           plain.flux_register().step_field(d))


def test_cache_recalls_the_choice(cuda, monkeypatch, tmp_path):
    monkeypatch.setenv("SNAPY_GB300_TUNE_CACHE", str(tmp_path / "sched.json"))
    a, _ = run(cuda, straka_vic(autotune=True), steps=1)
    b, _ = run(cuda, straka_vic(autotune=True), steps=1)
    assert a.batch.schedule["cached"] is False
    assert b.batch.schedule["cached"] is True
    assert a.batch.schedule["tj"] == b.batch.schedule["tj"]
    assert b.batch.tile(0) == a.batch.tile(0)


@pytest.mark.parametrize("tj", [1, 3, 8])
def test_every_schedule_gives_the_same_result(cuda, tj):
    """Tile widths and the two finish forms set through sg_set_schedule:
    the same state and step fields bit for bit."""
    out = []
    for finish in (1, 2):
        def sched(blk, vars, finish=finish):
            L = blk.batch.L
            t = (ctypes.c_int32 * 1)(tj)
            _lib.check(L.sg_set_schedule(blk.batch.h, t, finish), "sg_set_schedule")
            assert blk.batch.tile(0) == tj
        blk, vars = run(cuda, straka_vic(), before_steps=sched)
        out.append((vars["hydro_u"].clone(), blk.flux_register().step_field(1).clone()))
    ref, rv = run(cuda, straka_vic())
    for u, s1 in out:
        assert torch.equal(u, rv["hydro_u"])
        assert torch.equal(s1, ref.flux_register().step_field(1))
