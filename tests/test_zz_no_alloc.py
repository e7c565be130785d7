"""The allocation-free time-step entry point (sg_max_dt_noalloc).

Some callers cannot allocate device memory at all -- a host model that
hands the library views into its own arena, or a serving loop that admitted
a request against a fixed HBM budget.  This entry point computes the same
time steps as the handle path (sg_max_dt), keeping its reduction scratch in a
fixed __device__ array instead of a per-handle allocation.  The test calls it
through the C ABI and compares it with sg_max_dt on two calls in a row (the
second after the state moved on, so a stale scratch would show), in a fresh
process as well as after the other tests.
"""
import ctypes

import pytest
import torch

import snapy_gb300 as sg
from snapy_gb300 import _lib, problems

pytestmark = pytest.mark.gpu

MAX_BLOCKS = _lib.NOALLOC_MAX_BLOCKS
DtBlock = _lib.DtBlock


def _entry():
    L = _lib.load()
    return L, L.sg_max_dt_noalloc


def _blocks(cuda, decks):
    out = []
    for path, nx1, nx2, prec in decks:
        opts = sg.MeshBlockOptions.from_yaml(path)
        c = opts.coord()
        c.nx1, c.nx2 = nx1, nx2
        c.x1max, c.x2max = nx1 * 50.0, nx2 * 50.0
        opts.hydro().precision = prec
        blk = sg.MeshBlock(opts).to(cuda)
        vars = {"hydro_w": problems.straka(opts, cuda, xc=nx2 * 25.0, zc=nx1 * 25.0,
                                           xr=nx2 * 10.0, zr=nx1 * 10.0)}
        blk.initialize(vars)
        out.append((blk, vars))
    return out


def _noalloc_dt(fn, blk, cuda):
    b = blk.batch
    d = blk._block
    cur = b.current(0)
    arr = (DtBlock * 1)()
    a = arr[0]
    a.u = cur.data_ptr()
    a.nc1, a.nc2, a.nc3, a.ng = d["nc1"], d["nc2"], d["nc3"], d["ng"]
    a.dx1, a.dx2, a.dx3, a.gammad = d["dx1"], d["dx2"], d["dx3"], d["gammad"]
    nu = d.get("nu_iso", 0.0)
    a.dt_src = (min(d["dx1"], d["dx2"]) ** 2 / (2 * 2 * nu)) if nu > 0 else float("inf")
    a.implicit = int(d.get("implicit_scheme", 0))
    out = torch.full((1,), -1.0, dtype=torch.float64, device=cuda)
    dtype = 0 if blk.dtype == torch.float64 else 1
    rc = fn(arr, 1, dtype, blk.options.intg().cfl, b.redo.data_ptr(),
            out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == 0, _lib.load().sg_last_error().decode()
    return out.item()


def test_noalloc_matches_handle_path_twice(cuda):
    L, fn = _entry()
    cases = _blocks(cuda, [("snapy_gb300/decks/straka.yaml", 32, 48, "float64"),
                           ("snapy_gb300/decks/straka_noimplicit.yaml", 24, 40,
                            "float64")])
    for blk, vars in cases:
        for call in range(2):
            want = blk.max_time_step(vars)
            got = _noalloc_dt(fn, blk, cuda)
            assert got == pytest.approx(want, rel=1e-15), (call, got, want)
            blk.step(vars, 0.5 * want)  # the second call sees a new state


def test_noalloc_rejects_too_many_blocks(cuda):
    L, fn = _entry()
    arr = (DtBlock * (MAX_BLOCKS + 1))()
    out = torch.zeros(MAX_BLOCKS + 1, dtype=torch.float64, device=cuda)
    rc = fn(arr, MAX_BLOCKS + 1, 0, 0.9, None, out.data_ptr(),
            torch.cuda.current_stream().cuda_stream)
    assert rc != 0
    assert "SG_NOALLOC_MAX_BLOCKS" in L.sg_last_error().decode()
