"""The oracle's 3-D path (x3 faces, (x2, x3) columns of the implicit solve):
a state that does not vary along a periodic x3 steps exactly like its 2-D
slice (the x3 face fluxes are equal, their difference is zero)."""
import numpy as np
import pytest

import snapy_gb300 as sg
from snapy_gb300 import problems


def window(deck, nx1, nx2, nx3, cov=False, visc=False):
    opts = sg.MeshBlockOptions.from_yaml(f"snapy_gb300/decks/{deck}")
    c = opts.coord()
    c.nx1, c.nx2, c.nx3 = nx1, nx2, nx3
    c.x1max, c.x2max, c.x3max = nx1 * 50.0, nx2 * 50.0, nx3 * 50.0
    h = opts.hydro()
    if not visc:
        h.diffusion = None
    h.flux_covariance = cov
    if nx3 > 1:
        opts.bcnames = list(opts.bcnames[:4]) + ["periodic_inner", "periodic_outer"]
    return opts


@pytest.mark.parametrize("deck,cov,visc", [
    ("straka.yaml", False, False), ("straka_explicit.yaml", False, False),
    ("straka.yaml", True, False), ("straka_explicit.yaml", True, False),
    ("straka.yaml", True, True)])
def test_x3_uniform_3d_equals_2d(oracle, deck, cov, visc):
    """With the covariance row too (on x3 faces its u_n is zero), and with
    viscosity (the x3 derivatives vanish and the x3 faces' viscous fluxes are
    uniform along x3)."""
    o2 = window(deck, 24, 16, 1, cov, visc)
    o3 = window(deck, 24, 16, 6, cov, visc)
    if visc:
        assert o3.hydro().diffusion is not None and o3.hydro().diffusion.nu_iso > 0
    w2 = problems.straka(o2, "cpu", xc=300.0, zc=600.0, xr=300.0, zr=300.0).numpy()
    c3 = o3.coord()
    w3 = np.ascontiguousarray(np.broadcast_to(w2, (5, c3.nc3) + w2.shape[2:]))
    b2, b3 = oracle.block_from_options(o2), oracle.block_from_options(o3)
    u2, u3 = b2.initialize(w2), b3.initialize(w3)
    dt = 0.9 * min(b2.max_dt(u2), b3.max_dt(u3))
    for _ in range(3):
        for s in range(3):
            b2.stage(u2, dt, s)
            b3.stage(u3, dt, s)
    ng = c3.nghost
    for k in range(ng, c3.nc3 - ng):
        assert np.array_equal(u3[:, k], u2[:, 0]), k
