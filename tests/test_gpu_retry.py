"""The retry decision on the device (sg_check_retry): an ensemble in retry
mode ends every captured step with the check, and a rejected member gets
its step-start state back and half the dt, with no host read.  Each member
must follow the host-driven MeshBlock loop (max_time_step, step,
check_redo) bit for bit: the same states, redo counts and accepted time."""
import pytest
import torch

import snapy_gb300 as sg
from snapy_gb300 import problems
from snapy_gb300.ensemble import Ensemble

pytestmark = pytest.mark.gpu


def moving_sod(n, cfl, rho_r=None):
    opts = sg.MeshBlockOptions.from_yaml("snapy_gb300/decks/sod.yaml")
    opts.coord().nx1 = n
    opts.intg().cfl = cfl
    if rho_r is not None:
        opts.problem["rho_r"] = rho_r
    w = problems.sod(opts, "cpu")
    w[1] += 0.3
    return opts, w


def host_loop(opts, w, attempts, cuda):
    o = sg.MeshBlockOptions.from_yaml("snapy_gb300/decks/sod.yaml")
    o.coord().nx1 = opts.coord().nx1
    o.intg().cfl = opts.intg().cfl
    o.problem = dict(opts.problem)
    o.execution = "eager"
    o.autotune = False
    blk = sg.MeshBlock(o).to(cuda)
    vars = {"hydro_w": w.to(cuda)}
    blk.initialize(vars)
    t, redos, outcomes = 0.0, 0, []
    for _ in range(attempts):
        dt = blk.max_time_step(vars)
        blk.step(vars, dt)
        r = blk.check_redo(vars)
        outcomes.append(r)
        if r == 0:
            t += dt
        redos = blk.intg.current_redo
        if r < 0:
            break
    return vars["hydro_u"].clone(), redos, t, outcomes


def test_device_retry_follows_the_host_loop(cuda):
    members = [moving_sod(n, 4.0) for n in (128, 192, 256)]
    ens = Ensemble([o for o, _ in members], device=cuda, retry=True)
    ens.initialize([w for _, w in members], autotune=False)
    attempts = 8
    first = None
    for k in range(attempts):
        ens.step()
        if k == 0:
            first = ens.outcome.cpu().tolist()
    assert any(x == 1 for x in first), first  # the first attempts are rejected
    for k, (o, w) in enumerate(members):
        u, redo, t, outcomes = host_loop(o, w, attempts, cuda)
        assert outcomes[0] == 1
        assert torch.equal(ens.state(k), u), k
        assert int(ens.redo[k]) == redo
        assert float(ens.time[k]) == t
    assert ens.replays > 0


def test_a_member_past_max_redo_is_terminated_and_kept(cuda):
    """A member at the density floor is rejected at every attempt: past
    max_redo it is terminated, keeps its initial state and time 0, while
    the other member advances."""
    good = moving_sod(128, 0.4)
    bad = moving_sod(128, 0.4, rho_r=1.0005e-10)
    ens = Ensemble([good[0], bad[0]], device=cuda, retry=True)
    ens.initialize([good[1], bad[1]], autotune=False)
    u0 = ens.state(1).clone()
    max_redo = ens.max_redo
    for _ in range(max_redo + 3):
        ens.step()
    out = ens.outcome.cpu().tolist()
    assert out == [0, -1]
    assert torch.equal(ens.state(1), u0)
    assert float(ens.time[1]) == 0.0 and float(ens.time[0]) > 0.0
    _, redo, _, outcomes = host_loop(bad[0], bad[1], max_redo + 3, cuda)
    assert outcomes[-1] == -1 and int(ens.redo[1]) == redo
