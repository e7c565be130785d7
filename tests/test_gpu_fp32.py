"""FP32 bulk under gravity against the FP64 oracle.

An FP32 block with gravity stores its state as anomalies about an FP64
hydrostatic base, reconstructs and solves the Riemann problems in FP32 on
pressure anomalies, and keeps the hydrostatic reference, the base's balance
and the vertical implicit solve in FP64.  Its totals must stay within the
FP32 acceptance bar of the FP64 oracle on the same inputs and dt sequence:
relative L2 <= 1e-5 per conserved field.  The measured errors are printed.
"""
import numpy as np
import pytest
import torch

import snapy_gb300 as sg
from snapy_gb300 import problems

pytestmark = pytest.mark.gpu

TOL32 = 1e-5


def rel_l2(a, b):
    out = []
    for v in range(a.shape[0]):
        den = np.linalg.norm(b[v])
        num = np.linalg.norm(a[v] - b[v])
        out.append(num / den if den > 0 else num)
    return np.array(out)


def straka_window(deck, nx1, nx2, precision):
    opts = sg.MeshBlockOptions.from_yaml(f"snapy_gb300/decks/{deck}")
    c = opts.coord()
    c.nx1, c.nx2 = nx1, nx2
    c.x1max, c.x2max = nx1 * 50.0, nx2 * 50.0
    opts.hydro().precision = precision
    return opts


def interior(opts, u):
    c = opts.coord()
    ng = c.nghost
    return u[:, :, ng:c.nc2 - ng, ng:c.nc1 - ng]


@pytest.mark.parametrize("deck,iprec", [("straka_noimplicit.yaml", None),
                                        ("straka.yaml", "float64"),
                                        ("straka.yaml", "float32")])
def test_fp32_anomaly_against_fp64_oracle(oracle, cuda, deck, iprec):
    """iprec float32: the implicit blocks assembled in FP32 (the solve FP64)."""
    nx1, nx2, nstep, dt = 48, 64, 40, 0.1
    opts = straka_window(deck, nx1, nx2, "float32")
    if iprec:
        opts.hydro().icorr.precision = iprec
    blk = sg.MeshBlock(opts).to(cuda)
    assert blk.dtype == torch.float32
    w = problems.straka(opts, "cpu", xc=1600.0, zc=1200.0, xr=800.0, zr=600.0)
    vars = {"hydro_w": w.to(cuda)}
    blk.initialize(vars)
    ob = oracle.block_from_options(opts)
    u = ob.initialize(w.numpy())
    # the stored state is the anomaly; its totals start at the oracle's
    u0 = blk.total_u(vars).cpu().numpy()
    assert rel_l2(interior(opts, u0), interior(opts, u)).max() < 1e-7
    for step in range(nstep):
        blk.step(vars, dt)
        for s in range(3):
            ob.stage(u, dt, s)
    assert blk.check_redo(vars) == 0
    got = blk.total_u(vars).cpu().numpy()
    err = rel_l2(interior(opts, got), interior(opts, u))
    print(f"\n{deck} (implicit-precision {iprec}): FP32 anomaly vs FP64 oracle after {nstep} steps, "
          f"rel L2 per field (rho, m1, m2, m3, E): "
          + " ".join(f"{e:.2e}" for e in err))
    for v in (0, 1, 2, 4):
        assert err[v] <= TOL32, (v, err)


def test_fp32_anomaly_rest_state(cuda):
    """The base's balance is exact in FP64: an FP32 rest state stays at rest
    to FP32 roundoff of the anomalies."""
    opts = straka_window("straka.yaml", 64, 24, "float32")
    blk = sg.MeshBlock(opts).to(cuda)
    vars = {"hydro_w": problems.straka(opts, cuda, dT=0.0)}
    blk.initialize(vars)
    for _ in range(10):
        blk.step(vars, 0.1)
    vmax = blk.prim()[1:4].abs().max().item()
    print(f"\nFP32 rest state: max |v| after 10 steps {vmax:.2e} m/s")
    assert vmax < 1e-5


def test_fp32_anomaly_state_is_stored_about_the_base(cuda):
    opts = straka_window("straka_noimplicit.yaml", 32, 16, "float32")
    blk = sg.MeshBlock(opts).to(cuda)
    w = problems.straka(opts, cuda, xc=400.0, zc=800.0, xr=300.0, zr=300.0)
    vars = {"hydro_w": w.clone()}
    blk.initialize(vars)
    # the stored density is the anomaly about the base, the horizontal mean
    # of each x1 row: its row means vanish
    c = opts.coord()
    ng = c.nghost
    ra = vars["hydro_u"][0, 0, ng:c.nc2 - ng, ng:c.nc1 - ng].double()
    assert ra.mean(dim=0).abs().max().item() < 1e-7
    assert ra.abs().max().item() > 1e-3  # the bubble is in the anomaly
    tot = blk.total_u(vars)
    assert tot.dtype == torch.float64
    ref = w[0, 0, ng:c.nc2 - ng, ng:c.nc1 - ng]
    assert torch.allclose(tot[0, 0, ng:c.nc2 - ng, ng:c.nc1 - ng], ref, rtol=1e-7)
