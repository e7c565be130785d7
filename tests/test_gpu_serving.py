"""The serving loop: requests of different sizes admitted against an HBM
budget and advanced together.  Each request's result is the same alone and
in the mix (bit for bit: blocks never share tiles or columns), and a served
request equals the same deck stepped through MeshBlock."""
import pytest
import torch

import snapy_gb300 as sg
from snapy_gb300 import problems
from snapy_gb300.serving import Request, Server, footprint

pytestmark = pytest.mark.gpu


def conv(nx1, nx2, nx3, precision="float32"):
    opts = sg.MeshBlockOptions.from_yaml("snapy_gb300/decks/convection3d.yaml")
    c = opts.coord()
    c.nx1, c.nx2, c.nx3 = nx1, nx2, nx3
    c.x1max, c.x2max, c.x3max = nx1 * 50.0, nx2 * 50.0, nx3 * 50.0
    opts.hydro().precision = precision
    opts.problem["dtheta"] = 2.0
    opts.problem["layer"] = 0.4
    return opts


def request(rid, shape, seed, steps, arrival=0.0, precision="float32"):
    opts = conv(*shape, precision=precision)
    return Request(rid, opts, lambda: problems.convection3d(opts, "cpu", seed=seed),
                   steps, arrival)


SPECS = [(0, (24, 16, 12), 1, 6), (1, (32, 12, 16), 2, 4), (2, (24, 20, 12), 3, 5)]


def test_alone_equals_in_the_mix(cuda):
    mix = [request(rid, shape, seed, steps) for rid, shape, seed, steps in SPECS]
    # room for the first two only: the third waits for a completion
    budget = footprint(mix[0].options, torch.float32) + \
        footprint(mix[1].options, torch.float32)
    srv = Server(cuda, hbm_budget=budget)
    srv.run(mix)
    assert srv.max_running == 2
    assert srv.rebuilds >= 2
    assert mix[2].admitted >= mix[1].admitted
    for r in mix:
        assert r.flags == 0 and r.latency is not None and r.latency > 0
    for (rid, shape, seed, steps), r in zip(SPECS, mix):
        alone = request(rid, shape, seed, steps)
        Server(cuda).run([alone])
        assert torch.equal(alone.result, r.result), rid


def test_served_equals_meshblock(cuda):
    r = request(0, (24, 12, 10), 7, 5, precision="float64")
    Server(cuda).run([r])
    opts = conv(24, 12, 10, precision="float64")
    blk = sg.MeshBlock(opts).to(cuda)
    vars = {"hydro_w": problems.convection3d(opts, "cpu", seed=7).to(cuda)}
    blk.initialize(vars)
    for _ in range(5):
        blk.step(vars, blk.max_time_step(vars))
    assert torch.equal(vars["hydro_u"].cpu(), r.result)


def test_arrivals_are_served_in_order(cuda):
    reqs = [request(i, (16, 12, 12), 10 + i, 3, arrival=0.02 * i) for i in range(4)]
    srv = Server(cuda)
    srv.run(reqs)
    for a, b in zip(reqs, reqs[1:]):
        assert b.admitted >= a.admitted
    assert all(r.done >= r.admitted >= r.arrival for r in reqs)
    assert len(srv.gpu_step_ms) >= 3 and srv.launches > 0


def test_tracers_alone_equal_in_the_mix(cuda):
    """Requests whose deck carries a passive tracer: each one's tracer
    densities and state served alone equal those served in the mix, bit for
    bit."""
    import copy
    import numpy as np
    import snapy_gb300 as sg

    def tracer_request(rid, n, seed):
        cfg = copy.deepcopy(sg.options.yaml_lite.load(
            "snapy_gb300/decks/convection3d.yaml"))
        cfg["scalar"] = {"nvar": 1}
        cfg["dynamics"]["flux-covariance"] = False  # tracers: without it
        opts = sg.MeshBlockOptions.from_config(cfg)
        c = opts.coord()
        c.nx1, c.nx2, c.nx3 = n, 12, 10
        c.x1max, c.x2max, c.x3max = n * 50.0, 12 * 50.0, 10 * 50.0
        z = np.linspace(0.0, 1.0, c.nc1)[None, None, None, :]
        r = torch.from_numpy(1e-3 * (1.0 + 0.5 * np.sin(5.0 * z))
                             * np.ones((1, c.nc3, c.nc2, c.nc1)))
        return Request(rid, opts,
                       lambda: problems.convection3d(opts, "cpu", seed=seed), 4,
                       tracers=lambda: r)

    mix = [tracer_request(0, 16, 3), tracer_request(1, 24, 4)]
    Server(cuda).run(mix)
    for k, req in enumerate(mix):
        alone = tracer_request(9, 16 if k == 0 else 24, 3 + k)
        Server(cuda).run([alone])
        assert torch.equal(req.result, alone.result), k
        assert torch.equal(req.result_scalars, alone.result_scalars), k
