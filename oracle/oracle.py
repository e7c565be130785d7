"""ctypes binding of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Loads ``oracle/liboracle.so`` (the FP64 C restatement in ``sg_oracle.c``) and,
where it was built, ``oracle/_ref/libsnapref.so`` (the reference's own
header-only face kernels).  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU legs of ``bench.py`` import this module; the product package
``snapy_gb300`` never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libsnapref.so")

HLLC, LMARS = 0, 1
BC_NONE, BC_REFLECTING, BC_PERIODIC, BC_EXTRAPOLATION = 0, 1, 2, 3
BC_CODES = {
    "": BC_NONE,
    "none": BC_NONE,
    "custom": BC_NONE,
    "reflecting": BC_REFLECTING,
    "periodic": BC_PERIODIC,
    "extrapolation": BC_EXTRAPOLATION,
}

_dp = ctypes.POINTER(ctypes.c_double)


class OgBlock(ctypes.Structure):
    _fields_ = [
        ("nvar", ctypes.c_int),
        ("nc1", ctypes.c_int),
        ("nc2", ctypes.c_int),
        ("nc3", ctypes.c_int),
        ("ng", ctypes.c_int),
        ("dx1", ctypes.c_double),
        ("dx2", ctypes.c_double),
        ("dx3", ctypes.c_double),
        ("x1min", ctypes.c_double),
        ("x2min", ctypes.c_double),
        ("x3min", ctypes.c_double),
        ("gammad", ctypes.c_double),
        ("riemann", ctypes.c_int),
        ("shock", ctypes.c_int),
        ("weno_scale", ctypes.c_int),
        ("bc", ctypes.c_int * 6),
        ("wght", (ctypes.c_double * 3) * 3),
        ("nthreads", ctypes.c_int),
        ("grav1", ctypes.c_double),
        ("nu_iso", ctypes.c_double),
        ("flux_cov", ctypes.c_int),
        ("wb_wall_clamp", ctypes.c_int),
        ("implicit_scheme", ctypes.c_int),
        ("cfl", ctypes.c_double),
        ("x1f", _dp),
        ("x1v", _dp),
        ("x2v", _dp),
        ("step", _dp * 3),
        ("total", _dp * 3),
        ("nscalar", ctypes.c_int),
        ("scalar", _dp),
        ("scalar0", _dp),
        ("vic_q", _dp),
        ("monitor", ctypes.POINTER(ctypes.c_longlong)),
    ]


def build(quiet: bool = True) -> None:
    """Compile the oracle (and the reference shim when the reference exists)."""
    kw = dict(cwd=HERE, check=True)
    if quiet:
        kw.update(stdout=subprocess.DEVNULL)
    subprocess.run(["make", "-s", "all"], **kw)
    # the reference source tree: REFERENCE_ROOT, else the directory
    # "reference" beside the repository
    ref_root = os.environ.get("REFERENCE_ROOT") or os.path.abspath(
        os.path.join(HERE, "..", "..", "reference"))
    if os.path.isdir(os.path.join(ref_root, "src")):
        subprocess.run(["make", "-s", "ref", f"REFERENCE_ROOT={ref_root}"], **kw)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        L.og_weno5_face.restype = ctypes.c_double
        L.og_weno5_face.argtypes = [_dp, ctypes.c_int, ctypes.c_int]
        L.og_cp5_face.restype = ctypes.c_double
        L.og_cp5_face.argtypes = [_dp, ctypes.c_int]
        L.og_hllc_face.argtypes = [_dp, _dp, ctypes.c_double, ctypes.c_int, _dp, _dp]
        L.og_lmars_face.argtypes = [_dp, _dp, ctypes.c_double, ctypes.c_int, _dp, _dp]
        L.og_cons2prim_cell.argtypes = [_dp, _dp, ctypes.c_double, ctypes.c_int]
        bp = ctypes.POINTER(OgBlock)
        L.og_default_block.argtypes = [bp]
        L.og_cons2prim.argtypes = [bp, _dp, _dp]
        L.og_prim2cons.argtypes = [bp, _dp, _dp]
        L.og_apply_bc.argtypes = [bp, _dp, ctypes.c_int]
        L.og_scalar_bc.argtypes = [bp, _dp]
        L.og_flux.argtypes = [bp, _dp, ctypes.c_int, _dp]
        L.og_stage.argtypes = [bp, _dp, _dp, ctypes.c_double, ctypes.c_int]
        L.og_max_dt.restype = ctypes.c_double
        L.og_max_dt.argtypes = [bp, _dp]
        L.og_initialize.argtypes = [bp, _dp, _dp]
        L.og_tendency.argtypes = [bp, _dp, ctypes.c_double, _dp]
        L.og_implicit.restype = ctypes.c_int
        L.og_implicit.argtypes = [bp, _dp, ctypes.c_double, _dp]
        L.og_vic_redistribute_partial.argtypes = [ctypes.c_int, _dp, _dp, _dp, _dp]
        L.og_ref_column.argtypes = [bp, _dp, ctypes.c_size_t, _dp, _dp, _dp,
                                    _dp, _dp, _dp]
        L.og_recon_batch.argtypes = [_dp, ctypes.c_long, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int, _dp]
        L.og_shallow_roe_batch.argtypes = [_dp, _dp, ctypes.c_long, ctypes.c_int, _dp]
        L.og_hllc_sw_batch.argtypes = [_dp, _dp, ctypes.c_long, ctypes.c_int, _dp]
        _lib = L
    return _lib


def ref():
    """The reference's compiled header kernels, or None where not built."""
    global _ref
    if _ref is None and os.path.exists(REF_LIB):
        R = ctypes.CDLL(REF_LIB)
        R.ref_weno5_point.restype = ctypes.c_double
        R.ref_weno5_point.argtypes = [_dp, ctypes.c_int, ctypes.c_int]
        R.ref_cp5_point.restype = ctypes.c_double
        R.ref_cp5_point.argtypes = [_dp, ctypes.c_int]
        R.ref_hllc.argtypes = [_dp, _dp, _dp] + [ctypes.c_double] * 6 + [ctypes.c_int, _dp]
        R.ref_lmars.argtypes = [_dp, _dp, _dp] + [ctypes.c_double] * 4 + [ctypes.c_int, _dp]
        R.ref_shallow_roe.argtypes = [_dp, _dp, _dp, ctypes.c_int, ctypes.c_int]
        R.ref_cons2prim.argtypes = [_dp, _dp, ctypes.c_double]
        R.ref_pressure_scan.argtypes = [_dp, _dp, _dp, _dp, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_double]
        R.ref_hydro_ref_column.argtypes = [_dp, _dp, _dp, _dp, _dp, _dp, _dp,
                                           ctypes.c_int, ctypes.c_int,
                                           ctypes.c_double, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_int]
        _ref = R
    return _ref


def faces_linspace(xmin, dx, nc, ng=3):
    """Face coordinates of a padded axis as the reference builds them:
    torch.linspace(min - ng dx, max + ng dx, n + 2 ng + 1) in FP64 (callers
    with a deck pass the deck's own faces, CoordinateOptions.faces)."""
    import torch
    if nc <= 1:
        return np.array([xmin, xmin + dx])
    n = nc - 2 * ng
    xmax = xmin + n * dx
    return torch.linspace(xmin - ng * dx, xmax + ng * dx, nc + 1,
                          dtype=torch.float64).numpy()


def block_from_options(opts, nthreads=0):
    """An oracle block of a snapy_gb300 deck (options parsed by the product's
    reader; the geometry arrays come from the same linspace)."""
    c = opts.coord()
    h = opts.hydro()
    bcs = [n.rsplit("_", 1)[0] if n else "none" for n in opts.bcnames]
    bcs += ["none"] * (6 - len(bcs))
    g = h.grav.grav1 if h.grav else 0.0
    nu = h.diffusion.nu_iso if h.diffusion else 0.0
    return Block(nc1=c.nc1, nc2=c.nc2, nc3=c.nc3, dx1=c.dx1,
                 dx2=c.dx2 if c.nx2 > 1 else c.x2max - c.x2min,
                 dx3=c.dx3 if c.nx3 > 1 else c.x3max - c.x3min,
                 gammad=h.eos.gammad, riemann=h.riemann.type,
                 shock=h.recon1.shock, scale=h.recon1.scale, bc=bcs,
                 nthreads=nthreads, x1min=c.x1min, x2min=c.x2min,
                 x3min=c.x3min, grav1=g, nu_iso=nu,
                 flux_cov=h.flux_covariance, x1f=c.faces(1), x2f=c.faces(2),
                 implicit_scheme=h.icorr.scheme if h.icorr else 0,
                 cfl=opts.intg().cfl)


def vic_redistribute_partial(w: np.ndarray, du: np.ndarray, vol: np.ndarray,
                             delta: np.ndarray) -> np.ndarray:
    """The partial matrix's redistribution of one column (the constituent
    column, the tangential momenta carried by the face mass, the per-cell
    map): w, du (5, n); vol (n,); delta (n, 3).  Returns the new du."""
    w = np.ascontiguousarray(w, dtype=np.float64)
    out = np.array(du, dtype=np.float64, order="C")
    vol = np.ascontiguousarray(vol, dtype=np.float64)
    delta = np.ascontiguousarray(delta, dtype=np.float64)
    lib().og_vic_redistribute_partial(w.shape[1], ptr(w), ptr(out), ptr(vol),
                                      ptr(delta))
    return out


def ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


class Block:
    """An oracle block: the FP64 state and the reference's stage order."""

    def __init__(self, *, nc1, nc2=1, nc3=1, dx1=1.0, dx2=1.0, dx3=1.0,
                 gammad=1.4, riemann="hllc", shock=True, scale=False,
                 bc=("extrapolation",) * 6, nthreads=0, x1min=0.0, x2min=0.0,
                 x3min=0.0, grav1=0.0, nu_iso=0.0, flux_cov=True,
                 wb_wall_clamp=True, x1f=None, x2f=None, implicit_scheme=0,
                 cfl=0.9):
        L = lib()
        b = OgBlock()
        L.og_default_block(ctypes.byref(b))
        b.nvar = 5
        b.nc1, b.nc2, b.nc3 = nc1, nc2, nc3
        b.dx1, b.dx2, b.dx3 = dx1, dx2, dx3
        b.x1min, b.x2min, b.x3min = x1min, x2min, x3min
        b.gammad = gammad
        b.riemann = HLLC if riemann == "hllc" else LMARS
        b.shock = int(bool(shock))
        b.weno_scale = int(bool(scale))
        for f in range(6):
            b.bc[f] = BC_CODES[bc[f]] if isinstance(bc[f], str) else int(bc[f])
        b.nthreads = nthreads
        b.grav1, b.nu_iso = grav1, nu_iso
        b.flux_cov, b.wb_wall_clamp = int(bool(flux_cov)), int(bool(wb_wall_clamp))
        b.implicit_scheme = int(implicit_scheme)
        b.cfl = cfl
        # the reference's faces: a linspace over the padded extent
        # (CoordinateImpl::block_faces_, src/coord/coordinate.cpp:410-425)
        if x1f is None:
            x1f = faces_linspace(x1min, dx1, nc1)
        if x2f is None:
            x2f = faces_linspace(x2min, dx2, nc2)
        self.x1f = np.ascontiguousarray(x1f, dtype=np.float64)
        self.x1v = np.ascontiguousarray(0.5 * (self.x1f[:-1] + self.x1f[1:]))
        self.x2f = np.ascontiguousarray(x2f, dtype=np.float64)
        self.x2v = np.ascontiguousarray(0.5 * (self.x2f[:-1] + self.x2f[1:]))
        b.x1f, b.x1v, b.x2v = ptr(self.x1f), ptr(self.x1v), ptr(self.x2v)
        self.b = b
        self.shape = (5, nc3, nc2, nc1)
        self.u0 = np.zeros(self.shape)

    def initialize(self, w: np.ndarray) -> np.ndarray:
        w = np.ascontiguousarray(w, dtype=np.float64).copy()
        u = np.zeros(self.shape)
        lib().og_initialize(ctypes.byref(self.b), ptr(w), ptr(u))
        return u

    def prim(self, u: np.ndarray) -> np.ndarray:
        w = np.zeros(self.shape)
        lib().og_cons2prim(ctypes.byref(self.b), ptr(u), ptr(w))
        return w

    def max_dt(self, u: np.ndarray) -> float:
        return lib().og_max_dt(ctypes.byref(self.b), ptr(self.prim(u)))

    def stage(self, u: np.ndarray, dt: float, stage: int) -> None:
        lib().og_stage(ctypes.byref(self.b), ptr(u), ptr(self.u0), dt, stage)

    def step(self, u: np.ndarray, dt: float) -> None:
        for s in range(3):
            self.stage(u, dt, s)

    def tendency(self, w: np.ndarray, dt: float) -> np.ndarray:
        du = np.zeros(self.shape)
        lib().og_tendency(ctypes.byref(self.b), ptr(np.ascontiguousarray(w)), dt, ptr(du))
        return du

    def flux(self, w: np.ndarray, d: int) -> np.ndarray:
        f = np.zeros(self.shape)
        lib().og_flux(ctypes.byref(self.b), ptr(w), d, ptr(f))
        return f

    # -- the FluxRegister's step fields and register totals -----------------
    def request_step_field(self, dim: int) -> np.ndarray:
        """S_dim (FP64, zero), updated by every stage from here on."""
        if not hasattr(self, "_steps"):
            self._steps = [None, None, None]
        if self._steps[dim - 1] is None:
            self._steps[dim - 1] = np.zeros(self.shape)
            self.b.step[dim - 1] = ptr(self._steps[dim - 1])
        return self._steps[dim - 1]

    def step_field(self, dim: int) -> np.ndarray:
        return self._steps[dim - 1]

    # -- passive scalars (ScalarImpl, src/scalar/scalar.cpp:90-211) -----------
    def set_scalars(self, s: np.ndarray) -> np.ndarray:
        """Transport the tracer densities s (nscalar, nc3, nc2, nc1) with
        every stage from here on; returns the array the stages advance."""
        self._s = np.ascontiguousarray(s, dtype=np.float64).copy()
        self._s0 = np.zeros_like(self._s)
        self.b.nscalar = self._s.shape[0]
        self.b.scalar, self.b.scalar0 = ptr(self._s), ptr(self._s0)
        lib().og_scalar_bc(ctypes.byref(self.b), ptr(self._s))
        return self._s

    def count_monitor(self) -> np.ndarray:
        """The monitor count the stages raise from here on, [0] the interior
        faces whose HLLC contact pressure was clamped (riemann.pstar_clamp);
        returns the array the stages add into."""
        self._monitor = np.zeros(1, dtype=np.int64)
        self.b.monitor = self._monitor.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))
        return self._monitor

    def keep_totals(self, dim: int) -> np.ndarray:
        """The buffer each stage copies its register total T_dim into."""
        if not hasattr(self, "_totals"):
            self._totals = [None, None, None]
        if self._totals[dim - 1] is None:
            self._totals[dim - 1] = np.zeros(self.shape)
            self.b.total[dim - 1] = ptr(self._totals[dim - 1])
        return self._totals[dim - 1]


# ---------------------------------------------------------------------------
# the budget sums, restated (BudgetConsumer::totals and ::boundary,
# src/diagnostics/budget.cpp:68-155) -- the checker of the device sums
# ---------------------------------------------------------------------------
def _interior(b: OgBlock):
    out = []
    for n in (b.nc3, b.nc2, b.nc1):
        out.append(slice(b.ng, n - b.ng) if n > 1 else slice(0, 1))
    return tuple(out)


def budget_totals(blk: Block, u: np.ndarray) -> np.ndarray:
    """(5,) sum over the interior of u times the cell volume."""
    b = blk.b
    vol = b.dx3 * (b.dx2 * b.dx1)
    return np.array([(u[v][_interior(b)] * vol).sum() for v in range(5)])


def budget_boundary(blk: Block, steps) -> np.ndarray:
    """(5,) sum of sign A_f S_d on the reflecting and extrapolation faces of
    the interior cells (sign -1 lower, +1 upper)."""
    b = blk.b
    area = [b.dx3 * b.dx2, b.dx3 * b.dx1, b.dx2 * b.dx1]
    nc = [b.nc1, b.nc2, b.nc3]
    out = np.zeros(5)
    for d in range(3):
        S = steps[d] if d < len(steps) else None
        if S is None or nc[d] <= 1:
            continue
        for side in (0, 1):
            if b.bc[2 * d + side] not in (BC_REFLECTING, BC_EXTRAPOLATION):
                continue
            w = (1.0 if side else -1.0) * area[d]
            idx = list(_interior(b))
            ax = 2 - d  # (k, j, i) axis of direction d
            idx[ax] = nc[d] - b.ng if side else b.ng
            out += (S[(slice(None),) + tuple(idx)] * w).reshape(5, -1).sum(axis=1)
    return out
