"""Deck reading and the block's deck rules, on the CPU: every shipped deck
maps onto the stage, unknown keys and combinations outside the built scope
raise DeckError naming them, and there is no CPU path to fall back to."""
import copy
import glob
import os

import pytest

import snapy_gb300 as sg
from snapy_gb300 import yaml_lite
from snapy_gb300.meshblock import block_of, scheme_of
from snapy_gb300.options import DeckError

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DECKS = sorted(glob.glob(os.path.join(ROOT, "snapy_gb300", "decks", "*.yaml")))


def config(name):
    return yaml_lite.load(os.path.join(ROOT, "snapy_gb300", "decks", name))


def options(cfg):
    return sg.MeshBlockOptions.from_config(cfg, "deck.yaml")


@pytest.mark.parametrize("path", DECKS, ids=[os.path.basename(p) for p in DECKS])
def test_every_deck_maps_onto_the_stage(path):
    opts = sg.MeshBlockOptions.from_yaml(path)
    sch = scheme_of(opts)
    blk = block_of(opts)
    c = opts.coord()
    assert (blk["nc1"], blk["nc2"], blk["nc3"]) == (c.nc1, c.nc2, c.nc3)
    assert len(sch["wght"]) == 3 and len(blk["bc"]) == 6
    assert opts.execution in ("auto", "eager", "cuda-graph")
    assert opts.hydro().precision in ("float64", "float32")


def test_deck_values_reach_the_block():
    opts = options(config("straka.yaml"))
    blk = block_of(opts)
    assert blk["implicit_scheme"] == 9 and blk["grav1"] < 0
    assert blk["nu_iso"] == 75.0
    assert blk["nc1"] == 128 + 6 and blk["nc2"] == 512 + 6
    sod = options(config("sod.yaml"))
    assert scheme_of(sod)["shock"] and block_of(sod)["nc2"] == 1
    conv = options(config("convection3d.yaml"))
    assert conv.hydro().precision == "float32" and block_of(conv)["nc3"] > 1


@pytest.mark.parametrize("where,key", [((), "no-such-section"),
                                       (("integration",), "no-such-key"),
                                       (("dynamics",), "no-such-key")])
def test_unknown_keys_are_refused(where, key):
    cfg = copy.deepcopy(config("sod.yaml"))
    node = cfg
    for w in where:
        node = node[w]
    node[key] = 1
    with pytest.raises(DeckError, match=key):
        options(cfg)


def test_execution_keys():
    cfg = copy.deepcopy(config("sod.yaml"))
    cfg["integration"]["execution"] = "sometimes"
    with pytest.raises(DeckError, match="execution"):
        options(cfg)
    cfg["integration"]["execution"] = "eager"
    cfg["integration"]["execution-strict"] = True
    with pytest.raises(DeckError, match="execution-strict"):
        options(cfg)
    cfg = copy.deepcopy(config("sod.yaml"))
    cfg["integration"]["autotune"] = False
    assert options(cfg).autotune is False
    assert options(config("sod.yaml")).autotune is True


def _refused(cfg, match):
    with pytest.raises(DeckError, match=match):
        opts = options(cfg)
        scheme_of(opts)
        block_of(opts)


def test_fp32_under_gravity_needs_lmars():
    cfg = copy.deepcopy(config("straka.yaml"))
    cfg["dynamics"]["precision"] = "float32"
    cfg["dynamics"]["riemann-solver"]["type"] = "hllc"
    _refused(cfg, "lmars")


def test_fp32_implicit_assembly_needs_the_fp32_state():
    cfg = copy.deepcopy(config("straka.yaml"))
    cfg["integration"]["implicit-precision"] = "float32"
    _refused(cfg, "implicit-precision")


def test_3d_blocks_take_diffusion():
    """3-D blocks run the viscous fluxes of all three directions; what the
    diffusion section holds beyond nu_iso is refused by name."""
    cfg = copy.deepcopy(config("convection3d.yaml"))
    cfg.setdefault("forcing", {})["diffusion"] = {"nu_iso": 10.0}
    assert options(cfg).hydro().diffusion.nu_iso == 10.0
    cfg["forcing"]["diffusion"]["kappa_iso"] = 0.1
    _refused(cfg, "kappa_iso")


def test_refused_boundary_and_stencil():
    cfg = copy.deepcopy(config("sod.yaml"))
    cfg["boundary-condition"]["external"]["x1-inner"] = "outflow"
    _refused(cfg, "outflow")
    cfg = copy.deepcopy(config("sod.yaml"))
    cfg["geometry"]["cells"]["nghost"] = 2
    _refused(cfg, "nghost")


def test_no_cpu_path():
    opts = options(config("sod.yaml"))
    with pytest.raises(RuntimeError, match="CUDA"):
        sg.MeshBlock(opts).to("cpu")


def test_implicit_solve_keys():
    """integration.implicit-solve and implicit-corrections choose the solve
    of float32-assembled implicit blocks: sg_set_solve's argument."""
    cfg = copy.deepcopy(config("straka.yaml"))
    assert options(cfg).solve_corrections() == 2
    cfg["integration"]["implicit-corrections"] = 3
    assert options(cfg).solve_corrections() == 3
    cfg["integration"]["implicit-solve"] = "direct"
    assert options(cfg).solve_corrections() == 0
    for key, bad in (("implicit-solve", "float32"), ("implicit-corrections", 0),
                     ("implicit-corrections", 4)):
        cfg = copy.deepcopy(config("straka.yaml"))
        cfg["integration"][key] = bad
        with pytest.raises(DeckError, match=key):
            options(cfg)


def test_the_reference_import_name():
    """``import snapy`` is the drop-in's own surface."""
    import snapy
    import snapy_gb300
    assert snapy.MeshBlock is snapy_gb300.MeshBlock
    assert snapy.MeshBlockOptions is snapy_gb300.MeshBlockOptions
    assert (snapy.kIDN, snapy.kIPR) == (snapy_gb300.kIDN, snapy_gb300.kIPR)


def test_implicit_sweep_key():
    """integration/implicit-sweep: serial (default), partitioned or auto;
    a batch takes the serial sweep if any block asks for it."""
    from snapy_gb300.options import DeckError, MeshBlockOptions, shared_sweep
    base = {"geometry": {"type": "cartesian", "bounds": {"x1min": 0.0, "x1max": 1.0},
                         "cells": {"nx1": 16, "nghost": 3}},
            "dynamics": {"equation-of-state": {"type": "ideal-gas"},
                         "riemann-solver": {"type": "hllc"}},
            "integration": {"type": "rk3", "cfl": 0.4}}
    assert MeshBlockOptions.from_config(base).sweep_mode() == 0
    for name, mode in (("serial", 0), ("partitioned", 1), ("auto", 2)):
        cfg = dict(base, integration=dict(base["integration"], **{"implicit-sweep": name}))
        assert MeshBlockOptions.from_config(cfg).sweep_mode() == mode
    bad = dict(base, integration=dict(base["integration"], **{"implicit-sweep": "cyclic"}))
    with pytest.raises(DeckError):
        MeshBlockOptions.from_config(bad)
    assert shared_sweep([1, 1]) == 1
    assert shared_sweep([1, 2]) == 2
    assert shared_sweep([2, 0, 1]) == 0
