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
    "outflow": BC_EXTRAPOLATION,
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
    ]


def build(quiet: bool = True) -> None:
    """Compile the oracle (and the reference shim when the reference exists)."""
    kw = dict(cwd=HERE, check=True)
    if quiet:
        kw.update(stdout=subprocess.DEVNULL)
    subprocess.run(["make", "-s", "all"], **kw)
    ref_root = os.environ.get("REFERENCE_ROOT", "/root/reference")
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
        L.og_flux.argtypes = [bp, _dp, ctypes.c_int, _dp]
        L.og_stage.argtypes = [bp, _dp, _dp, ctypes.c_double, ctypes.c_int]
        L.og_max_dt.restype = ctypes.c_double
        L.og_max_dt.argtypes = [bp, _dp]
        L.og_initialize.argtypes = [bp, _dp, _dp]
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
        _ref = R
    return _ref


def ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


class Block:
    """An oracle block: the FP64 state and the reference's stage order."""

    def __init__(self, *, nc1, nc2=1, nc3=1, dx1=1.0, dx2=1.0, dx3=1.0,
                 gammad=1.4, riemann="hllc", shock=True, scale=False,
                 bc=("extrapolation",) * 6, nthreads=0, x1min=0.0, x2min=0.0,
                 x3min=0.0):
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

    def flux(self, w: np.ndarray, d: int) -> np.ndarray:
        f = np.zeros(self.shape)
        lib().og_flux(ctypes.byref(self.b), ptr(w), d, ptr(f))
        return f
