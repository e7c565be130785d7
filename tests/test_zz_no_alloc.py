"""The allocation-free time-step entry point (sg_max_dt_noalloc).

Some callers cannot allocate device memory at all -- a host model that
hands the library views into its own arena, or a serving loop that admitted
a request against a fixed HBM budget.  This entry point computes the same
time steps as the handle path (sg_max_dt), keeping its reduction scratch in a
fixed __device__ array instead of a per-handle allocation.

The tests call it through the C ABI and compare it with the handle path:
* on two calls in a row, the second after the state moved on (a stale
  scratch would show);
* for the header's documented inputs: dt_src = 0 for "no bound", the deck's
  implicit-scheme number (9) for the vertical solve;
* for FP32 blocks that hold anomalies about an FP64 hydrostatic base;
* for one call over several blocks of different sizes with a nonzero redo
  count per block;
* once more in a fresh process, where the first call of the process looks
  the scratch's address up.
"""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import pytest  # noqa: E402
import torch  # noqa: E402

import snapy_gb300 as sg  # noqa: E402
from snapy_gb300 import _lib, problems  # noqa: E402

pytestmark = pytest.mark.gpu

MAX_BLOCKS = _lib.NOALLOC_MAX_BLOCKS
DtBlock = _lib.DtBlock
TOL = 1e-15

# (deck, nx1, nx2, precision): implicit FP64 with viscosity, explicit FP64,
# implicit FP32 (anomalies about the hydrostatic base), explicit FP32
DECKS = [("snapy_gb300/decks/straka.yaml", 32, 48, "float64"),
         ("snapy_gb300/decks/straka_noimplicit.yaml", 24, 40, "float64"),
         ("snapy_gb300/decks/straka.yaml", 40, 56, "float32"),
         ("snapy_gb300/decks/straka_noimplicit.yaml", 16, 72, "float32")]


def _entry():
    L = _lib.load()
    return L, L.sg_max_dt_noalloc


def _block(cuda, deck, nx1, nx2, prec):
    opts = sg.MeshBlockOptions.from_yaml(os.path.join(ROOT, deck))
    c = opts.coord()
    c.nx1, c.nx2 = nx1, nx2
    c.x1max, c.x2max = nx1 * 50.0, nx2 * 50.0
    opts.hydro().precision = prec
    blk = sg.MeshBlock(opts).to(cuda)
    vars = {"hydro_w": problems.straka(opts, cuda, xc=nx2 * 25.0, zc=nx1 * 25.0,
                                       xr=nx2 * 10.0, zr=nx1 * 10.0)}
    blk.initialize(vars)
    return blk, vars


def _describe(blk, a):
    """Fill one sg_dt_block the way the header documents it."""
    b = blk.batch
    d = blk._block
    a.u = b.current(0).data_ptr()
    a.nc1, a.nc2, a.nc3, a.ng = d["nc1"], d["nc2"], d["nc3"], d["ng"]
    a.dx1, a.dx2, a.dx3, a.gammad = d["dx1"], d["dx2"], d["dx3"], d["gammad"]
    nu = d.get("nu_iso", 0.0)
    ndim = sum(1 for n in (d["nc1"], d["nc2"], d["nc3"]) if n > 1)
    # 0 is the header's "no bound"
    a.dt_src = (min(d["dx1"], d["dx2"]) ** 2 / (2 * ndim * nu)) if nu > 0 else 0.0
    a.implicit = int(d.get("implicit_scheme", 0))  # the scheme number: 9
    base = b.bases[0]
    a.base = base.data_ptr() if base is not None else None


def _call(fn, blks, redo, cuda):
    arr = (DtBlock * len(blks))()
    for a, blk in zip(arr, blks):
        _describe(blk, a)
    out = torch.full((len(blks),), -1.0, dtype=torch.float64, device=cuda)
    red = torch.tensor(redo, dtype=torch.int32, device=cuda)
    dtype = 0 if blks[0].dtype == torch.float64 else 1
    rc = fn(arr, len(blks), dtype, blks[0].options.intg().cfl, red.data_ptr(),
            out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == 0, _lib.load().sg_last_error().decode()
    return out.tolist()


def test_noalloc_matches_handle_path_twice(cuda):
    L, fn = _entry()
    for deck in DECKS:
        blk, vars = _block(cuda, *deck)
        for call in range(2):
            want = blk.max_time_step(vars)
            got = _call(fn, [blk], [0], cuda)[0]
            assert got == pytest.approx(want, rel=TOL), (deck, call, got, want)
            blk.step(vars, 0.5 * want)  # the second call sees a new state


@pytest.mark.parametrize("prec", ["float64", "float32"])
def test_noalloc_several_blocks_with_redo(cuda, prec):
    """One call over blocks of different sizes (the grid covers the largest,
    blockIdx.y picks the block), each with its own redo count."""
    L, fn = _entry()
    cases = [_block(cuda, d, nx1, nx2, p) for d, nx1, nx2, p in DECKS if p == prec]
    cases.append(_block(cuda, "snapy_gb300/decks/straka.yaml", 64, 96, prec))
    redo = [0, 2, 1][:len(cases)]
    for call in range(2):
        want = [blk.max_time_step(vars) * 2.0 ** -r
                for (blk, vars), r in zip(cases, redo)]
        got = _call(fn, [blk for blk, _ in cases], redo, cuda)
        for g, w in zip(got, want):
            assert g == pytest.approx(w, rel=TOL), (call, got, want)
        for blk, vars in cases:
            blk.step(vars, 0.5 * blk.max_time_step(vars))


def test_noalloc_rejects_too_many_blocks(cuda):
    L, fn = _entry()
    arr = (DtBlock * (MAX_BLOCKS + 1))()
    out = torch.zeros(MAX_BLOCKS + 1, dtype=torch.float64, device=cuda)
    rc = fn(arr, MAX_BLOCKS + 1, 0, 0.9, None, out.data_ptr(),
            torch.cuda.current_stream().cuda_stream)
    assert rc != 0
    assert "SG_NOALLOC_MAX_BLOCKS" in L.sg_last_error().decode()


def test_noalloc_rejects_base_on_fp64(cuda):
    L, fn = _entry()
    blk, _ = _block(cuda, *DECKS[0])
    arr = (DtBlock * 1)()
    _describe(blk, arr[0])
    arr[0].base = blk.batch.current(0).data_ptr()  # any device pointer
    out = torch.zeros(1, dtype=torch.float64, device=cuda)
    rc = fn(arr, 1, 0, 0.9, None, out.data_ptr(),
            torch.cuda.current_stream().cuda_stream)
    assert rc != 0
    assert "base" in L.sg_last_error().decode()


def test_noalloc_in_a_fresh_process(cuda):
    """The first call of a process looks the scratch's address up: run the
    two-call comparison in a new interpreter."""
    env = dict(os.environ)
    r = subprocess.run([sys.executable, os.path.abspath(__file__)], cwd=ROOT,
                       env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "noalloc fresh process ok" in r.stdout


if __name__ == "__main__":
    dev = torch.device("cuda", 0)
    test_noalloc_matches_handle_path_twice(dev)
    print("noalloc fresh process ok")
