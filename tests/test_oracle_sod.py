"""The oracle on the 1-D Sod tube: the known solution's features and exact
mass conservation (extrapolation ends, no flux through them by t = 0.2)."""
import numpy as np


def sod_oracle(O, nx=256):
    ng, nc1, dx = 3, nx + 6, 1.0 / nx
    b = O.Block(nc1=nc1, dx1=dx, riemann="hllc", shock=True,
                bc=("extrapolation",) * 6)
    x = (np.arange(nc1) - ng + 0.5) * dx
    w = np.zeros((5, 1, 1, nc1))
    w[0] = np.where(x < 0.5, 1.0, 0.125)
    w[4] = np.where(x < 0.5, 1.0, 0.1)
    return b, b.initialize(w), x


def test_sod_to_t02(oracle):
    b, u, x = sod_oracle(oracle)
    m0 = u[0, 0, 0, 3:-3].sum()
    t = 0.0
    while t < 0.2:
        dt = 0.4 * b.max_dt(u)
        dt = min(dt, 0.2 - t)
        b.step(u, dt)
        t += dt
    w = b.prim(u)[:, 0, 0, 3:-3]
    xi = x[3:-3]
    # shock between 0.84 and 0.86, contact near 0.69, rarefaction head 0.26
    jump = np.argmax(np.abs(np.diff(w[0])) * (xi[:-1] > 0.8))
    assert 0.84 < xi[jump] < 0.86
    assert abs(w[2].max()) == 0.0 and abs(w[3].max()) == 0.0
    plateau = w[4][(xi > 0.55) & (xi < 0.8)]
    assert np.allclose(plateau, 0.30313, rtol=2e-2)
    assert abs(u[0, 0, 0, 3:-3].sum() - m0) <= 1e-13 * m0


def test_oracle_straka_rest_is_balanced(oracle):
    """The well-balanced x1 reference: a resting isentropic column has a
    tendency at round-off (momentum) with gravity, viscosity and the
    covariance row on."""
    import snapy_gb300 as sg
    from snapy_gb300 import problems
    opts = sg.MeshBlockOptions.from_yaml("snapy_gb300/decks/straka_noimplicit.yaml")
    c = opts.coord()
    c.nx1, c.nx2, c.x1max, c.x2max = 64, 16, 3200.0, 800.0
    ob = oracle.block_from_options(opts)
    u = ob.initialize(problems.straka(opts, "cpu", dT=0.0).numpy())
    du = ob.tendency(ob.prim(u), 1.0)
    assert np.abs(du[1]).max() < 1e-11 * np.abs(u[0]).max() * 9.8
    assert np.abs(du[2]).max() == 0.0
