"""The drop-in surface's smaller pieces: ``import snapy`` (the reference's
import name) and MeshBlock.module(name).buffer(name) (python/csrc/
pyoptions.hpp:99-116)."""
import pytest
import torch

import snapy
import snapy_gb300 as sg
from snapy_gb300 import problems

pytestmark = pytest.mark.gpu


def test_module_buffers(cuda):
    opts = snapy.MeshBlockOptions.from_yaml("snapy_gb300/decks/straka.yaml")
    c = opts.coord()
    c.nx1, c.nx2, c.x1max, c.x2max = 24, 32, 24 * 50.0, 32 * 50.0
    opts.hydro().precision = "float32"
    blk = snapy.MeshBlock(opts).to(cuda)
    vars = {"hydro_w": problems.straka(opts, cuda)}
    blk.initialize(vars)
    assert blk.module("hydro").buffer("hydro_u").data_ptr() == vars["hydro_u"].data_ptr()
    x1f = blk.module("coord").buffer("x1f")
    assert x1f.shape == (c.nc1 + 1,) and x1f.dtype == torch.float64
    assert torch.allclose(blk.buffer("x1v"), 0.5 * (x1f[:-1] + x1f[1:]))
    assert blk.buffer("hydro_ref").shape == (5 * c.nc1 + 1,)
    before = vars["hydro_u"].clone()
    blk.forward(vars, blk.max_time_step(vars), 0)
    # after stage 0 the backup u0 holds the step's input
    assert torch.equal(blk.module("hydro").buffer("u0"), before)
    with pytest.raises(KeyError):
        blk.module("chemistry")
    with pytest.raises(KeyError):
        blk.module("coord").buffer("hydro_u")
