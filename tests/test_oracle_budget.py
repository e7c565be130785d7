"""The oracle's FluxRegister step fields and budget sums (CPU).

The step-field recursion S_d <- w1 S_d + w2 dt T_d against the closed
product form sum_s w2_s prod_{t>s} w1_t dt T_s, as the reference's
tests/test_flux_register.cpp:211-249 checks it (bar 1e-15 of max |sum|),
and the budget closing: with no sources, change + boundary = 0 per row."""
import numpy as np
import pytest

import snapy_gb300 as sg
from snapy_gb300 import problems

RK3 = [[1.0, 0.0, 1.0], [0.75, 0.25, 0.25], [1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0]]


def straka_window(deck, nx1, nx2):
    opts = sg.MeshBlockOptions.from_yaml(deck)
    c = opts.coord()
    c.nx1, c.nx2 = nx1, nx2
    c.x1max, c.x2max = nx1 * 50.0, nx2 * 50.0
    return opts


@pytest.mark.parametrize("deck", ["snapy_gb300/decks/straka_noimplicit.yaml",
                                  "snapy_gb300/decks/straka.yaml"])
def test_step_field_recursion_equals_the_weighted_stage_sum(oracle, deck):
    opts = straka_window(deck, 24, 16)
    ob = oracle.block_from_options(opts)
    w = problems.straka(opts, "cpu", xc=400.0, zc=600.0, xr=300.0, zr=300.0)
    u = ob.initialize(w.numpy())
    S = [ob.request_step_field(d) for d in (1, 2)]
    T = [ob.keep_totals(d) for d in (1, 2)]
    worst = 0.0
    for step in range(5):
        dt = 0.9 * ob.max_dt(u)
        Ts = []
        for s in range(3):
            ob.stage(u, dt, s)
            Ts.append([t.copy() for t in T])
        for d in range(2):
            ref = np.zeros_like(S[d])
            for s in range(3):
                c = RK3[s][2]
                for t in range(s + 1, 3):
                    c *= RK3[t][1]
                ref += (c * dt) * Ts[s][d]
            scale = np.abs(ref).max()
            assert scale > 0
            rel = np.abs(S[d] - ref).max() / scale
            worst = max(worst, rel)
            assert rel <= 1e-15, (step, d + 1, rel)
    print(f"\nstep fields: worst max|S - sum c_s dt T_s| / max|sum| = {worst:.3e}")


def test_implicit_posts_enter_the_x1_total(oracle):
    """The implicit solve posts its face transfers into T_1: the mass row
    differs from the explicit flux on interior faces, and the wall faces'
    mass and energy rows stay prescribed (zero)."""
    opts = straka_window("snapy_gb300/decks/straka.yaml", 24, 16)
    ob = oracle.block_from_options(opts)
    w = problems.straka(opts, "cpu", xc=400.0, zc=600.0, xr=300.0, zr=300.0)
    u = ob.initialize(w.numpy())
    T1 = ob.keep_totals(1)
    dt = 0.9 * ob.max_dt(u)
    ob.stage(u.copy(), dt, 0)
    imp = T1.copy()
    ob.b.implicit_scheme = 0
    ob.stage(u.copy(), dt, 0)
    exp = T1.copy()
    ng, nc1 = 3, opts.coord().nc1
    assert np.abs(imp[0] - exp[0]).max() > 0
    assert np.array_equal(imp[1], exp[1])  # the normal momentum gets no post
    for f in (ng, nc1 - ng):
        assert not imp[0][..., f].any() and not imp[4][..., f].any()


def moving_sod(oracle, n=128, vx=0.3):
    opts = sg.MeshBlockOptions.from_yaml("snapy_gb300/decks/sod.yaml")
    opts.coord().nx1 = n
    ob = oracle.block_from_options(opts)
    w = problems.sod(opts, "cpu")
    w[1] += vx  # mass, momentum and energy cross both ends
    return opts, ob, w.numpy()


def test_budget_closes_without_sources(oracle):
    opts, ob, w = moving_sod(oracle)
    u = ob.initialize(w)
    S1 = ob.request_step_field(1)
    start = oracle.budget_totals(ob, u)
    pending = np.zeros(5)
    for _ in range(40):
        dt = 0.4 * ob.max_dt(u)
        ob.step(u, dt)
        pending += oracle.budget_boundary(ob, [S1])
    change = oracle.budget_totals(ob, u) - start
    scale = np.abs(start) + np.abs(pending)
    assert np.abs(pending[[0, 1, 4]]).min() > 0  # mass, momentum, energy cross
    assert np.all(np.abs(change + pending) <= 1e-13 * scale), (change, pending)


def test_budget_walls_carry_no_mass(oracle):
    """Reflecting walls all round: the mass and energy rows of the boundary
    transfer are zero, the x1 momentum row is the pressure on the walls, and
    the mass total does not change beyond roundoff."""
    opts = straka_window("snapy_gb300/decks/straka_noimplicit.yaml", 24, 16)
    ob = oracle.block_from_options(opts)
    w = problems.straka(opts, "cpu", xc=400.0, zc=600.0, xr=300.0, zr=300.0)
    u = ob.initialize(w.numpy())
    S = [ob.request_step_field(1), ob.request_step_field(2)]
    start = oracle.budget_totals(ob, u)
    pending = np.zeros(5)
    for _ in range(5):
        ob.step(u, 0.9 * ob.max_dt(u))
        pending += oracle.budget_boundary(ob, S)
    assert pending[0] == 0.0 and pending[4] == 0.0
    assert pending[1] != 0.0
    change = oracle.budget_totals(ob, u) - start
    assert abs(change[0]) <= 1e-14 * abs(start[0])
