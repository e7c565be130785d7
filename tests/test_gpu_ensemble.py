"""Batched ensembles: members of uneven size in one launch per stage.

Each member's result is the same alone and in the batch (bit for bit in
FP64: every tile computes its own faces from its own block's data, whatever
else shares the launch)."""
import pytest
import torch

import snapy_gb300 as sg
from snapy_gb300 import problems
from snapy_gb300.ensemble import Ensemble

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("deck", ["straka_noimplicit.yaml", "straka.yaml"])
def test_member_alone_equals_member_in_batch(cuda, deck):
    members = problems.ensemble_members(n=3, seed=7, deck=deck,
                                        nx2_choices=(24, 40, 56),
                                        nx1_choices=(32, 48))
    ens = Ensemble([m for m, _ in members], device=cuda)
    ens.initialize([w for _, w in members])
    # the buffer rotation at the start of a step runs (0,0), (1,0), (0,1),
    # (1,0), ...: steps 1-3 run eagerly, step 4 on is captured and replayed
    nstep = 6
    for _ in range(nstep):
        ens.step()
    torch.cuda.synchronize()
    for k, (opts, w) in enumerate(members):
        blk = sg.MeshBlock(opts).to(cuda)
        vars = {"hydro_w": w.to(cuda)}
        blk.initialize(vars)
        for _ in range(nstep):
            dt = blk.max_time_step(vars)
            blk.step(vars, dt)
        assert torch.equal(vars["hydro_u"], ens.state(k)), k
    assert ens.replays == 3 and ens.captures == 2


def test_ensemble_flags_one_member(cuda):
    """A NaN planted in one member flags that member only."""
    members = problems.ensemble_members(n=3, seed=3, deck="straka_noimplicit.yaml",
                                        nx2_choices=(24, 40), nx1_choices=(32,))
    ens = Ensemble([m for m, _ in members], device=cuda)
    ens.initialize([w for _, w in members])
    ens.step()
    ens.state(1)[0, 0, 10, 10] = float("nan")
    flags = ens.check()
    assert flags[1].item() & 8 and flags[0].item() == 0 and flags[2].item() == 0
