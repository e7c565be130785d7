"""The oracle's partial matrix (implicit-scheme 1: the 3x3 blocks of rows and
columns {rho, m1, E}, the tangential momenta folded into the density column
and carried by the face mass transfers), on the CPU.

* The reference's own known-answer property of the redistribution
  (tests/test_backward_substitution.cpp:308-365): a uniform tangential wind
  stays uniform, each tangential momentum's column sum is unchanged, and a
  wind-free column's tangential rows are untouched bit for bit (a signed
  zero survives).
* Whole blocks: a resting isentropic column stays at rest, mass is
  conserved in the closed box, and the solution is close to the full
  matrix's (the two differ only in how the tangential momenta are solved).
"""
import copy

import numpy as np
import pytest

import snapy_gb300 as sg
from snapy_gb300 import problems

IDN, IVX, IVY, IVZ, IPR = range(5)


@pytest.mark.parametrize("wind", [True, False])
def test_tangential_momentum_follows_the_face_mass(oracle, wind):
    n = 4
    v2, v3 = 400.0, -30.0
    vol = np.array([1.0, 2.0, 1.5, 0.5])
    rho = np.array([3.0, 2.5, 4.0, 1.8])
    corr = np.array([0.4, -0.2, 0.1, -0.3])
    w = np.zeros((5, n))
    du = np.zeros((5, n))
    w[IDN] = rho
    w[IVY] = v2 if wind else 0.0
    w[IVZ] = v3 if wind else 0.0
    du[IVY] = -0.0  # a signed zero must survive
    delta = np.zeros((n, 3))
    delta[:, 0] = corr
    out = oracle.vic_redistribute_partial(w, du, vol, delta)
    if not wind:
        for v in (IVY, IVZ):
            assert np.array_equal(out[v], du[v])
            assert np.array_equal(np.signbit(out[v]), np.signbit(du[v]))
        return
    for v in (IVY, IVZ):
        assert abs((out[v] * vol).sum()) <= 1e-12
    rho1 = rho + out[IDN]
    assert np.all(out[IDN] != 0.0)
    assert np.allclose((rho * v2 + out[IVY]) / rho1, v2, rtol=0, atol=1e-12)
    assert np.allclose((rho * v3 + out[IVZ]) / rho1, v3, rtol=0, atol=1e-12)


def straka(scheme, nx1=40, nx2=48, dT=-15.0, dx2=50.0):
    cfg = copy.deepcopy(sg.options.yaml_lite.load("snapy_gb300/decks/straka.yaml"))
    cfg["integration"]["implicit-scheme"] = scheme
    opts = sg.MeshBlockOptions.from_config(cfg)
    c = opts.coord()
    c.nx1, c.nx2, c.x1max, c.x2max = nx1, nx2, nx1 * 50.0, nx2 * dx2
    w = problems.straka(opts, "cpu", dT=dT, xc=1200.0, zc=1000.0, xr=600.0,
                        zr=500.0).numpy()
    return opts, w


def run(oracle, opts, w, nsteps, dt_scale=1.0):
    ob = oracle.block_from_options(opts)
    u = ob.initialize(w)
    dt = dt_scale * ob.max_dt(u)
    for _ in range(nsteps):
        ob.step(u, dt)
    return ob, u


@pytest.mark.parametrize("scheme", [1, 9])
def test_rest_state_stays_at_rest(oracle, scheme):
    """A resting isentropic column (no bubble) with x2 cells 40 times the
    x1 ones, so the implicit-aware CFL step puts the vertical acoustic
    Courant number near 40: the velocities stay at round-off."""
    opts, w = straka(scheme, nx1=48, nx2=8, dT=0.0, dx2=2000.0)
    ob, u = run(oracle, opts, w, 10)
    wf = ob.prim(u)[:, 0, 3:-3, 3:-3]
    assert np.isfinite(u).all()
    print(f"scheme {scheme}: max |v1| {np.abs(wf[IVX]).max():.2e}, "
          f"max |v2| {np.abs(wf[IVY]).max():.2e}")
    assert np.abs(wf[IVX]).max() < 1e-8
    assert np.abs(wf[IVY]).max() < 1e-8


def test_partial_conserves_mass_and_is_close_to_full(oracle):
    """The bubble window for 6 steps at the implicit-aware CFL step: the partial
    matrix conserves mass in the closed box to round-off, moves the state,
    and stays close to the full matrix's solution."""
    opts1, w = straka(1)
    opts9, _ = straka(9)
    ob1, u1 = run(oracle, opts1, w, 6)
    _, u9 = run(oracle, opts9, w, 6)
    u0 = ob1.initialize(w)
    inner = (slice(3, -3), slice(3, -3))
    m0 = u0[IDN][0][inner].sum()
    assert abs(u1[IDN][0][inner].sum() - m0) <= 1e-13 * m0
    assert not np.array_equal(u1, u0)
    for v in range(5):
        a, b = u1[v][0][inner], u9[v][0][inner]
        scale = max(np.abs(b).max(), 1e-300)
        rel = np.abs(a - b).max() / scale
        print(f"var {v}: max |scheme 1 - scheme 9| / max |scheme 9| = {rel:.2e}")
        assert rel < 1e-3


def test_deck_accepts_scheme_1():
    opts, _ = straka(1)
    sg.meshblock.scheme_of(opts)
    assert sg.meshblock.block_of(opts)["implicit_scheme"] == 1
    cfg = copy.deepcopy(sg.options.yaml_lite.load("snapy_gb300/decks/straka.yaml"))
    cfg["integration"]["implicit-scheme"] = 1
    cfg["integration"]["implicit-precision"] = "float32"
    cfg["dynamics"]["precision"] = "float32"
    opts = sg.MeshBlockOptions.from_config(cfg)
    sg.meshblock.scheme_of(opts)  # FP32 assembly, as for scheme 9
    d = sg.meshblock.block_of(opts)
    assert d["implicit_scheme"] == 1 and d["implicit_f32"]
    cfg["integration"]["implicit-scheme"] = 5
    with pytest.raises(sg.options.DeckError, match="scheme 1"):
        sg.meshblock.scheme_of(sg.MeshBlockOptions.from_config(cfg))
