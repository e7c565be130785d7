"""The oracle's passive-scalar transport (ScalarImpl::forward,
src/scalar/scalar.cpp:90-211) against the properties the reference's own
scalar tests hold (tests/test_tracer_ratio.py's no-limiter arm: a uniform
ratio stays uniform to round-off; tests/test_scalar.cpp: ds finite, the
tracer moves with the flow), plus conservation in a closed box; and the
deck's scalar section, with what is not built refused by name."""
import copy

import numpy as np
import pytest

import snapy_gb300 as sg
from snapy_gb300 import problems
from snapy_gb300.options import DeckError
from oracle import oracle


def straka_explicit(nx1=32, nx2=48, deck="straka_noimplicit.yaml", cov=False):
    cfg = copy.deepcopy(sg.options.yaml_lite.load("snapy_gb300/decks/" + deck))
    cfg["dynamics"]["flux-covariance"] = cov
    opts = sg.MeshBlockOptions.from_config(cfg)
    c = opts.coord()
    c.nx1, c.nx2, c.x1max, c.x2max = nx1, nx2, nx1 * 50.0, nx2 * 50.0
    return opts


def run(nsteps=10, deck="straka_noimplicit.yaml", cov=False):
    opts = straka_explicit(deck=deck, cov=cov)
    ob = oracle.block_from_options(opts)
    w = problems.straka(opts, "cpu", xc=1000.0, zc=1200.0, xr=800.0,
                        zr=600.0).numpy()
    u = ob.initialize(w)
    c = opts.coord()
    i = np.arange(c.nc1)[None, None, :]
    r = np.stack([np.full(u[0].shape, 0.37), np.where(i > 16, 2.0, 0.0) + 0 * u[0]])
    s = ob.set_scalars(u[0] * r)
    vol = ob.b.dx1 * ob.b.dx2 * ob.b.dx3
    inner = (slice(None), slice(3, -3), slice(3, -3))
    m0 = [s[v][inner].sum() * vol for v in range(2)]
    top0 = s[1][inner][..., 16:].sum()
    for _ in range(nsteps):
        ob.step(u, ob.max_dt(u))
    return ob, u, s, m0, vol, inner, top0


@pytest.mark.parametrize("cov", [False, True])
@pytest.mark.parametrize("deck", ["straka_noimplicit.yaml", "straka.yaml"])
def test_uniform_ratio_conservation_and_transport(deck, cov):
    """Explicit, and with the vertical implicit solve (the tracer's share of
    its dry transfer, donor-capped); without and with the flux-covariance
    row, whose scalar row and positivity limiter keep the stepped tracer
    non-negative."""
    ob, u, s, m0, vol, inner, top0 = run(deck=deck, cov=cov)
    assert np.isfinite(s).all()
    if cov:
        assert s[1][inner].min() >= 0.0
    ratio = s[0][inner] / u[0][inner]
    assert np.abs(ratio / 0.37 - 1).max() <= 1e-13
    for v in range(2):
        assert abs(s[v][inner].sum() * vol - m0[v]) <= 1e-13 * abs(m0[v])
    # the step in the second tracer is carried by the flow
    assert s[1][inner][..., 16:].sum() != top0


def test_deck_scalar_section():
    cfg = sg.options.yaml_lite.load("snapy_gb300/decks/straka_noimplicit.yaml")
    cfg = copy.deepcopy(cfg)
    cov = copy.deepcopy(cfg)
    cov["scalar"] = {"nvar": 1}
    # with the covariance row (the default): the scalar's row and the
    # positivity limiter are built
    assert sg.MeshBlockOptions.from_config(cov).scalar_names == ["scalar0"]
    cfg["dynamics"]["flux-covariance"] = False
    cfg["scalar"] = {"nvar": 1, "names": ["tracer"]}
    assert sg.MeshBlockOptions.from_config(cfg).scalar_names == ["tracer"]
    cfg["scalar"] = {"nvar": 2}
    assert sg.MeshBlockOptions.from_config(cfg).scalar_names == ["scalar0", "scalar1"]
    for extra, word in ((("upper-bound", 1.0), "upper-bound"),
                        (("riemann-solver", {"type": "hllc"}), "upwind")):
        bad = copy.deepcopy(cfg)
        bad["scalar"][extra[0]] = extra[1]
        with pytest.raises(DeckError, match=word):
            sg.MeshBlockOptions.from_config(bad)
    d3 = copy.deepcopy(sg.options.yaml_lite.load("snapy_gb300/decks/convection3d.yaml"))
    d3["scalar"] = {"nvar": 1}
    assert sg.MeshBlockOptions.from_config(d3).scalar_names == ["scalar0"]
    d3["dynamics"]["flux-covariance"] = False
    assert sg.MeshBlockOptions.from_config(d3).scalar_names == ["scalar0"]
