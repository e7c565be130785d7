"""The C ABI refuses what it does not build, loudly: each call returns its
error code (SG_ERR_ARG 1, SG_ERR_UNSUPPORTED 3) and names the reason in
sg_last_error, and no handle is left behind."""
import ctypes

import pytest
import torch

import snapy_gb300 as sg
from snapy_gb300 import _lib

pytestmark = pytest.mark.gpu

ARG, UNSUPPORTED = 1, 3
RK3 = [[1.0, 0.0, 1.0], [0.75, 0.25, 0.25], [1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0]]


def scheme(dtype=_lib.F64, riemann=_lib.HLLC):
    s = _lib.Scheme()
    s.dtype, s.riemann, s.shock, s.scale, s.nstage = dtype, riemann, 1, 0, 3
    for i in range(3):
        for j in range(3):
            s.wght[i][j] = RK3[i][j]
    s.cfl, s.density_floor, s.pressure_floor = 0.4, 1e-10, 1e-10
    return s


def block(nc1=38, nc2=1, nc3=1, ng=3, **kw):
    b = _lib.BlockDesc()
    b.nc1, b.nc2, b.nc3, b.ng = nc1, nc2, nc3, ng
    for f in range(6):
        b.bc[f] = _lib.BC_EXTRAPOLATION
    b.dx1 = b.dx2 = b.dx3 = 1.0
    b.gammad, b.flux_cov, b.wb_wall_clamp = 1.4, 0, 1
    for k, v in kw.items():
        if k == "bc":
            for f in range(6):
                b.bc[f] = v[f]
        else:
            setattr(b, k, v)
    return b


def create(sch, blk):
    L = _lib.load()
    h = ctypes.c_void_p()
    rc = L.sg_create(ctypes.byref(sch), (_lib.BlockDesc * 1)(blk), 1, ctypes.byref(h))
    msg = L.sg_last_error().decode()
    if rc == 0:
        L.sg_destroy(h)
    return rc, h.value, msg


def geometry(cuda, nc1):
    f = torch.linspace(-3.0, nc1 - 3.0, nc1 + 1, dtype=torch.float64, device=cuda)
    return f, 0.5 * (f[1:] + f[:-1]).contiguous()


def test_create_refuses_what_is_not_built(cuda):
    f, v = geometry(cuda, 38)
    walls = [_lib.BC_REFLECTING] * 2 + [_lib.BC_EXTRAPOLATION] * 4
    grav = dict(grav1=-9.8, x1f=f.data_ptr(), x1v=v.data_ptr(), bc=walls)
    base = torch.zeros(5 * 38 + 1, dtype=torch.float64, device=cuda)
    cases = [
        (scheme(), block(ng=2), UNSUPPORTED, "nghost"),
        (scheme(), block(nc1=6), ARG, "sizes"),
        (scheme(), block(implicit_scheme=9), UNSUPPORTED, "const-gravity"),
        (scheme(), block(implicit_scheme=7, **grav), UNSUPPORTED, "scheme 9"),
        (scheme(_lib.F32, _lib.LMARS), block(**grav), ARG, "base"),
        (scheme(_lib.F32, _lib.HLLC), block(base=base.data_ptr(), **grav),
         UNSUPPORTED, "lmars"),
        (scheme(), block(base=base.data_ptr(), **grav), ARG, "base"),
        (scheme(), block(implicit_precision=_lib.F32), UNSUPPORTED,
         "implicit-precision"),
        (scheme(), block(bc=[9] * 6), ARG, "boundary kind"),
        (scheme(), block(grav1=-9.8), ARG, "x1 geometry"),
    ]
    for sch, blk, code, word in cases:
        rc, h, msg = create(sch, blk)
        assert (rc, word in msg) == (code, True), (word, rc, msg)
    # a valid block still builds, and implicit-scheme 1 assembles in FP32 as
    # scheme 9 does (an FP32 state under gravity: LMARS, about its base)
    assert create(scheme(), block())[0] == 0
    rc, _, msg = create(scheme(_lib.F32, _lib.LMARS),
                        block(implicit_scheme=1, implicit_precision=_lib.F32,
                              base=base.data_ptr(), **grav))
    assert rc == 0, msg


def test_step_fields_need_their_direction_and_scratch(cuda):
    L = _lib.load()
    opts = sg.MeshBlockOptions.from_yaml("snapy_gb300/decks/sod.yaml")
    b = sg.MeshBlock(opts).to(cuda).batch
    s = torch.zeros(b.shapes[0], dtype=torch.float64, device=cuda)
    assert L.sg_bind_step_fields(b.h, 0, None, s.data_ptr(), None, None, 0) == ARG
    assert "x2" in L.sg_last_error().decode()
    # an implicit block's x1 field needs the staging scratch
    opts = sg.MeshBlockOptions.from_yaml("snapy_gb300/decks/straka.yaml")
    c = opts.coord()
    c.nx1, c.nx2, c.x1max, c.x2max = 16, 8, 800.0, 400.0
    b = sg.MeshBlock(opts).to(cuda).batch
    s = torch.zeros(b.shapes[0], dtype=torch.float64, device=cuda)
    assert L.sg_bind_step_fields(b.h, 0, s.data_ptr(), None, None, None, 0) == ARG
    assert "scratch" in L.sg_last_error().decode()


def test_cubed_sphere_fp32_index_limit(cuda):
    """The FP32 handle's tables carry flat indices in FP32: a grid with 2^24
    faces or more is refused before anything is read."""
    L = _lib.load()
    dummy = torch.zeros(16, dtype=torch.float64, device=cuda)
    d = _lib.CsDesc()
    d.n, d.ng, d.dtype, d.nstage = 1700, 3, _lib.F32, 3
    d.geo = d.ghost_tab = d.seam_tab = d.seam_state_tab = dummy.data_ptr()
    d.nghost, d.nseam, d.phi_ref, d.cfl = 1, 1, 9810.0, 0.4
    d.nseam_state = 24 * d.n
    h = ctypes.c_void_p()
    assert L.sg_cs_create(ctypes.byref(d), ctypes.byref(h)) == UNSUPPORTED
    assert "2^24" in L.sg_last_error().decode() and not h.value
