"""The serving admission's device-byte count (no GPU): the state buffers,
the implicit solve's scratch (with the refined solve's FP32 part for
FP32-assembled blocks) and the passive scalars' buffers and face scratch."""
import copy

import torch

import snapy_gb300 as sg
from snapy_gb300.serving import footprint


def deck(scalars=0, precision="float32", implicit_precision="float32"):
    cfg = copy.deepcopy(sg.options.yaml_lite.load("snapy_gb300/decks/convection3d.yaml"))
    if scalars:
        cfg["scalar"] = {"nvar": scalars}
        cfg["dynamics"]["flux-covariance"] = False  # tracers: without it
    opts = sg.MeshBlockOptions.from_config(cfg)
    opts.hydro().precision = precision
    opts.hydro().icorr.precision = implicit_precision
    return opts


def test_footprint_counts_each_part():
    base = deck()
    c = base.coord()
    nc = c.nc1 * c.nc2 * c.nc3
    icells = c.nx1 * c.nx2 * c.nx3
    plain = footprint(deck(implicit_precision="float64"), torch.float32)
    refined = footprint(base, torch.float32)
    # the refined solve's FP32 part: 160 floats per cell, 7 per column
    assert refined - plain == (icells * 160 + (icells // c.nx1) * 7) * 4 + 16
    # two tracers: three FP32 buffers each and the FP64 face scratch
    two = footprint(deck(scalars=2), torch.float32)
    assert two - refined == 3 * 2 * nc * 4 + (4 + 5 * 2) * nc * 8
