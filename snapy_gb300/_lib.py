"""ctypes binding of ``libsnapy_gb300.so`` (the C ABI in include/snapy_gb300.h).

The library is the only compute path of this package: if it is missing and
cannot be built (no nvcc), importing the binding raises instead of falling
back to anything else.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

_i32 = ctypes.c_int32
_dp = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p

F64, F32 = 0, 1
HLLC, LMARS = 0, 1
BC_NONE, BC_REFLECTING, BC_PERIODIC, BC_EXTRAPOLATION = 0, 1, 2, 3


class Scheme(ctypes.Structure):
    _fields_ = [
        ("dtype", _i32),
        ("riemann", _i32),
        ("shock", _i32),
        ("scale", _i32),
        ("nstage", _i32),
        ("wght", (ctypes.c_double * 3) * 3),
        ("cfl", ctypes.c_double),
        ("density_floor", ctypes.c_double),
        ("pressure_floor", ctypes.c_double),
    ]


class BlockDesc(ctypes.Structure):
    _fields_ = [
        ("nc1", _i32),
        ("nc2", _i32),
        ("nc3", _i32),
        ("ng", _i32),
        ("bc", _i32 * 6),
        ("dx1", ctypes.c_double),
        ("dx2", ctypes.c_double),
        ("dx3", ctypes.c_double),
        ("gammad", ctypes.c_double),
        ("tj", _i32),
        ("grav1", ctypes.c_double),
        ("nu_iso", ctypes.c_double),
        ("flux_cov", _i32),
        ("wb_wall_clamp", _i32),
        ("x1f", _vp),
        ("x1v", _vp),
        ("implicit_scheme", _i32),
        ("base", _vp),
        ("implicit_precision", _i32),
        ("nscalar", _i32),
    ]


class DtBlock(ctypes.Structure):
    """sg_dt_block: one block of the allocation-free time step."""
    _fields_ = [("u", _vp), ("nc1", _i32), ("nc2", _i32), ("nc3", _i32),
                ("ng", _i32), ("dx1", ctypes.c_double), ("dx2", ctypes.c_double),
                ("dx3", ctypes.c_double), ("gammad", ctypes.c_double),
                ("dt_src", ctypes.c_double), ("implicit", _i32),
                ("base", _vp)]


NOALLOC_MAX_BLOCKS = 64  # SG_NOALLOC_MAX_BLOCKS

# SG_KERNEL_* of sg_kernel_times
KERNELS = ("stage_kernel", "vic_assemble_kernel", "vic_solve_kernel",
           "vic_finish_kernel", "ghost_kernel", "x3_kernel", "scalar_kernel")


class CsDesc(ctypes.Structure):
    """sg_cs_desc: the cubed-sphere handle's grid, scheme and tables."""
    _fields_ = [("n", _i32), ("ng", _i32), ("dtype", _i32), ("nstage", _i32),
                ("wght", (ctypes.c_double * 3) * 3), ("cfl", ctypes.c_double),
                ("geo", _vp), ("ghost_tab", _vp), ("nghost", _i32),
                ("seam_tab", _vp), ("nseam", _i32), ("phi_ref", ctypes.c_double),
                ("riemann", _i32), ("seam_state_tab", _vp), ("nseam_state", _i32)]


# every symbol include/snapy_gb300.h declares, with its ctypes signature
SIGNATURES = {
    "sg_create": (ctypes.c_int, [ctypes.POINTER(Scheme), ctypes.POINTER(BlockDesc),
                                 _i32, ctypes.POINTER(_vp)]),
    "sg_destroy": (ctypes.c_int, [_vp]),
    "sg_bind": (ctypes.c_int, [_vp, _i32, _vp, _vp, _vp]),
    "sg_scratch_bytes": (ctypes.c_int, [_vp, _i32, ctypes.POINTER(ctypes.c_size_t)]),
    "sg_bind_scratch": (ctypes.c_int, [_vp, _i32, _vp, ctypes.c_size_t]),
    "sg_set_current": (ctypes.c_int, [_vp, _i32]),
    "sg_current": (ctypes.c_int, [_vp, ctypes.POINTER(_i32)]),
    "sg_rotation": (ctypes.c_int, [_vp, ctypes.POINTER(_i32), ctypes.POINTER(_i32)]),
    "sg_set_rotation": (ctypes.c_int, [_vp, _i32, _i32]),
    "sg_advance": (ctypes.c_int, [_vp, _i32]),
    "sg_stage": (ctypes.c_int, [_vp, _i32, _vp, _vp]),
    "sg_fill_ghosts": (ctypes.c_int, [_vp, _vp]),
    "sg_max_dt": (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    "sg_check": (ctypes.c_int, [_vp, _vp, _vp]),
    "sg_init_from_prim": (ctypes.c_int, [_vp, ctypes.POINTER(_vp), _vp]),
    "sg_restore": (ctypes.c_int, [_vp]),
    "sg_prim": (ctypes.c_int, [_vp, ctypes.POINTER(_vp), _vp]),
    "sg_tile": (ctypes.c_int, [_vp, _i32, ctypes.POINTER(_i32)]),
    "sg_launches_per_stage": (ctypes.c_int, [_vp, ctypes.POINTER(_i32)]),
    "sg_step_scratch_bytes": (ctypes.c_int, [_vp, _i32, ctypes.POINTER(ctypes.c_size_t)]),
    "sg_bind_step_fields": (ctypes.c_int, [_vp, _i32, _vp, _vp, _vp, _vp, ctypes.c_size_t]),
    "sg_budget_totals": (ctypes.c_int, [_vp, _vp, _vp]),
    "sg_budget_boundary": (ctypes.c_int, [_vp, _vp, _i32, _vp]),
    "sg_set_solve": (ctypes.c_int, [_vp, _i32]),
    "sg_bind_scalars": (ctypes.c_int, [_vp, _i32, _vp, _vp, _vp]),
    "sg_solve_fallbacks": (ctypes.c_int, [_vp, _vp]),
    "sg_set_sweep": (ctypes.c_int, [_vp, _i32]),
    "sg_sweep": (ctypes.c_int, [_vp, ctypes.POINTER(_i32)]),
    "sg_psw_rcp": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, _vp]),
    "sg_add_step_counts": (ctypes.c_int, [_vp, _vp, _vp]),
    "sg_autotune": (ctypes.c_int, [_vp, _i32, _vp, _vp, _vp, _vp]),
    "sg_set_schedule": (ctypes.c_int, [_vp, _vp, _i32]),
    "sg_check_retry": (ctypes.c_int, [_vp, _vp, _vp, _i32, _vp, _vp]),
    "sg_set_timing": (ctypes.c_int, [_vp, _i32]),
    "sg_kernel_times": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_double),
                                       ctypes.POINTER(ctypes.c_int64)]),
    "sg_last_error": (ctypes.c_char_p, []),
    "sg_version": (ctypes.c_char_p, []),
    "sg_max_dt_noalloc": (ctypes.c_int, [ctypes.POINTER(DtBlock), _i32, _i32,
                                         ctypes.c_double, _vp, _vp, _vp]),
    "sg_cs_create": (ctypes.c_int, [ctypes.POINTER(CsDesc), ctypes.POINTER(_vp)]),
    "sg_cs_destroy": (ctypes.c_int, [_vp]),
    "sg_cs_scratch_bytes": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_size_t)]),
    "sg_cs_bind": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, ctypes.c_size_t]),
    "sg_cs_set_current": (ctypes.c_int, [_vp, _i32]),
    "sg_cs_rotation": (ctypes.c_int, [_vp, ctypes.POINTER(_i32), ctypes.POINTER(_i32)]),
    "sg_cs_set_rotation": (ctypes.c_int, [_vp, _i32, _i32]),
    "sg_cs_advance": (ctypes.c_int, [_vp, _i32]),
    "sg_cs_stage": (ctypes.c_int, [_vp, _i32, _vp, _vp]),
    "sg_cs_fill_seams": (ctypes.c_int, [_vp, _vp]),
    "sg_cs_max_dt": (ctypes.c_int, [_vp, _vp, _vp]),
    "sg_cs_bind_step_fields": (ctypes.c_int, [_vp, _vp, _vp]),
    "sg_cs_budget_totals": (ctypes.c_int, [_vp, _vp, _vp]),
}

_lib = None
_lock = threading.Lock()


class SgError(RuntimeError):
    pass


def load(build_if_missing: bool = True):
    """Load the CUDA library (building it in-tree first when it is stale)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if build_if_missing and not _build.up_to_date():
            try:
                _build.build()
            except Exception as e:  # no nvcc: the CUDA path cannot exist
                if not os.path.exists(path):
                    raise SgError(
                        "snapy_gb300: libsnapy_gb300.so is missing and could "
                        f"not be built ({e}); run __graft_entry__.build()") from e
        if not os.path.exists(path):
            raise SgError("snapy_gb300: libsnapy_gb300.so is missing; run "
                          "__graft_entry__.build()")
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return L


def check(rc: int, what: str = "") -> None:
    if rc != 0:
        msg = load().sg_last_error().decode()
        raise SgError(f"{what}: {msg} (code {rc})" if what else f"{msg} (code {rc})")
