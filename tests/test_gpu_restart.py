"""Resume from a restart file: a run interrupted by write_restart and
continued by a fresh block's initialize_from_restart equals the run that was
never interrupted, bit for bit (FP64; FP32 stored as anomalies about the
FP64 hydrostatic base, with the refined implicit solve; with a passive
tracer), and the restored time, cycle and file checks are the reference's
(src/mesh/meshblock_restart.cpp:33-236)."""
import copy

import pytest
import torch

import snapy_gb300 as sg
from snapy_gb300 import problems, restart as R

pytestmark = pytest.mark.gpu


def straka(precision, implicit=True, tracer=False):
    deck = "straka.yaml" if implicit else "straka_noimplicit.yaml"
    cfg = copy.deepcopy(sg.options.yaml_lite.load(f"snapy_gb300/decks/{deck}"))
    if tracer:
        cfg["scalar"] = {"nvar": 1}
        cfg["dynamics"]["flux-covariance"] = False
    opts = sg.MeshBlockOptions.from_config(cfg)
    c = opts.coord()
    c.nx1, c.nx2, c.x1max, c.x2max = 40, 48, 40 * 50.0, 48 * 50.0
    opts.hydro().precision = precision
    if precision == "float32" and implicit:
        opts.hydro().icorr.precision = "float32"
    return opts


def start(opts, cuda):
    blk = sg.MeshBlock(opts).to(cuda)
    vars = {"hydro_w": problems.straka(opts, cuda, xc=1200.0, zc=1000.0,
                                       xr=600.0, zr=500.0)}
    if opts.scalar_names:
        c = opts.coord()
        z = torch.linspace(0.0, 1.0, c.nc1, dtype=torch.float64, device=cuda)
        vars["scalar_r"] = (1e-3 * (1.0 + 0.5 * torch.sin(5.0 * z))).expand(
            1, c.nc3, c.nc2, c.nc1).contiguous()
    blk.initialize(vars)
    return blk, vars


def run(blk, vars, n, t):
    for _ in range(n):
        dt = blk.max_time_step(vars)
        blk.step(vars, dt)
        assert blk.check_redo(vars) == 0
        blk.cycle += 1
        t += dt
    return t


@pytest.mark.parametrize("precision, implicit, tracer", [
    ("float64", True, False), ("float32", True, False), ("float64", False, True)])
def test_resume_equals_the_uninterrupted_run(cuda, tmp_path, precision, implicit,
                                             tracer):
    opts = straka(precision, implicit, tracer)
    blk, vars = start(opts, cuda)
    t = run(blk, vars, 4, 0.0)
    path = blk.write_restart(vars, str(tmp_path), basename="straka", number=1,
                             time=t)
    assert path.endswith("straka.00001.restart")
    t_end = run(blk, vars, 4, t)
    fresh = sg.MeshBlock(opts).to(cuda)
    v2 = {}
    t2 = fresh.initialize_from_restart(v2, path)
    assert t2 == t and fresh.cycle == 4
    t2_end = run(fresh, v2, 4, t2)
    assert t2_end == t_end
    assert torch.equal(v2["hydro_u"], vars["hydro_u"])
    if tracer:
        assert torch.equal(v2["scalar_s"], vars["scalar_s"])
    data = R.load_restart(path)
    if precision == "float32":
        # the file holds totals; the stored bits and the base ride along
        assert data["hydro_u"].dtype == torch.float64
        assert data["hydro_u_stored"].dtype == torch.float32
        assert data[R.HYDRO_RESTART_METADATA].tolist() == [1, 32]
    else:
        assert R.HYDRO_RESTART_METADATA not in data


def test_resume_refuses_another_grid(cuda, tmp_path):
    opts = straka("float32")
    blk, vars = start(opts, cuda)
    path = blk.write_restart(vars, str(tmp_path), basename="g", time=0.0)
    other = straka("float32")
    c = other.coord()
    c.x1max = c.x1max * 1.5  # the same shape on other faces
    with pytest.raises(R.RestartError, match="reference grid mismatch"):
        sg.MeshBlock(other).to(cuda).initialize_from_restart({}, path)
