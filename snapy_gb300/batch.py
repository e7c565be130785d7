"""A batch of blocks advanced together by the CUDA library.

``Batch`` owns one library handle, the three rotating HBM state buffers of
every block (torch allocations, handed to the library as raw pointers) and the
per-block device time steps.  ``MeshBlock`` is a batch of one; an ensemble or
the serving loop batches many blocks of one scheme into one launch per stage.
"""
from __future__ import annotations

import ctypes
from typing import List, Optional, Sequence

import torch

from . import _lib

_DT = {torch.float64: _lib.F64, torch.float32: _lib.F32}


def _stream(stream: Optional[torch.cuda.Stream] = None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def fill_base(t: torch.Tensor, w: torch.Tensor, d: dict) -> None:
    """The FP64 hydrostatic base of an anomaly block (sg_block_desc.base)
    from its initial primitives w: the horizontal mean of rho and p on each
    x1 row, e_b = p_b / (gamma - 1), face pressures pf_b (mean of the two
    cells beside a face, end faces copy the end cells) and the base's
    residual r_b = rho_b g1 - (pf_b[i + 1] - pf_b[i]) / dx1.  Any base gives
    the same equations; one near the state keeps the FP32 anomalies small."""
    nc1, nc2, nc3, ng = d["nc1"], d["nc2"], d["nc3"], d["ng"]
    j = slice(ng, nc2 - ng) if nc2 > 1 else slice(0, 1)
    k = slice(ng, nc3 - ng) if nc3 > 1 else slice(0, 1)
    rho = w[0, k, j, :].mean(dim=(0, 1))
    pres = w[4, k, j, :].mean(dim=(0, 1))
    pf = torch.empty(nc1 + 1, dtype=torch.float64, device=w.device)
    pf[1:nc1] = 0.5 * (pres[:-1] + pres[1:])
    pf[0], pf[nc1] = pres[0], pres[-1]
    r = rho * d["grav1"] - (pf[1:] - pf[:-1]) / d["dx1"]
    t[0:nc1] = rho
    t[nc1:2 * nc1] = pres
    t[2 * nc1:3 * nc1] = pres / (d["gammad"] - 1.0)
    t[3 * nc1:4 * nc1 + 1] = pf
    t[4 * nc1 + 1:5 * nc1 + 1] = r


class Batch:
    """Blocks of one scheme; each block is a dict with nc1, nc2, nc3, ng,
    dx1, dx2, dx3, gammad, bc (6 ints) and optionally tj."""

    def __init__(self, scheme: dict, blocks: Sequence[dict],
                 device: torch.device, dtype: torch.dtype):
        if device.type != "cuda":
            raise RuntimeError("snapy_gb300 runs on CUDA devices only "
                               f"(got {device}); there is no CPU path")
        self.L = _lib.load()
        self.device = device
        self.dtype = dtype
        self.nblock = len(blocks)
        self.scheme_key = [int(scheme["riemann"]), int(bool(scheme["shock"])),
                           int(bool(scheme["scale"]))]
        self.schedule = None  # the autotuner's choice, once tuned
        self.sweep_mode = 0  # sg_set_sweep's mode (0: the serial sweep)
        sch = _lib.Scheme()
        sch.dtype = _DT[dtype]
        sch.riemann = scheme["riemann"]
        sch.shock = int(scheme["shock"])
        sch.scale = int(scheme["scale"])
        sch.nstage = len(scheme["wght"])
        for s, w in enumerate(scheme["wght"]):
            for q in range(3):
                sch.wght[s][q] = w[q]
        sch.cfl = scheme["cfl"]
        sch.density_floor = scheme["density_floor"]
        sch.pressure_floor = scheme["pressure_floor"]
        arr = (_lib.BlockDesc * self.nblock)()
        # FP64 x1 geometry per block on the device (kept alive here)
        self.geom = []
        for d in blocks:
            f = torch.as_tensor(d["x1f"], dtype=torch.float64, device=device) \
                if d.get("x1f") is not None else None
            v = torch.as_tensor(d["x1v"], dtype=torch.float64, device=device) \
                if d.get("x1v") is not None else None
            self.geom.append((f, v))
        for b, d in enumerate(blocks):
            a = arr[b]
            a.nc1, a.nc2, a.nc3, a.ng = d["nc1"], d["nc2"], d["nc3"], d["ng"]
            for f in range(6):
                a.bc[f] = d["bc"][f]
            a.dx1, a.dx2, a.dx3 = d["dx1"], d["dx2"], d["dx3"]
            a.gammad = d["gammad"]
            a.tj = d.get("tj", 0)
            a.grav1 = d.get("grav1", 0.0)
            a.nu_iso = d.get("nu_iso", 0.0)
            a.flux_cov = int(bool(d.get("flux_cov", True)))
            a.wb_wall_clamp = int(bool(d.get("wb_wall_clamp", True)))
            f, v = self.geom[b]
            a.x1f = f.data_ptr() if f is not None else None
            a.x1v = v.data_ptr() if v is not None else None
            a.implicit_scheme = int(d.get("implicit_scheme", 0))
            a.implicit_precision = _lib.F32 if d.get("implicit_f32") else _lib.F64
            a.nscalar = int(d.get("nscalar", 0))
        # FP32 under gravity: the state is stored as anomalies about an FP64
        # hydrostatic base per block (filled from the initial state)
        self.bases = []
        for b, d in enumerate(blocks):
            t = None
            if dtype == torch.float32 and d.get("grav1", 0.0) != 0.0:
                t = torch.zeros(5 * d["nc1"] + 1, dtype=torch.float64, device=device)
                arr[b].base = t.data_ptr()
            self.bases.append(t)
        self.blocks = [dict(d) for d in blocks]
        self.shapes = [(5, d["nc3"], d["nc2"], d["nc1"]) for d in blocks]
        h = ctypes.c_void_p()
        with torch.cuda.device(device):
            _lib.check(self.L.sg_create(ctypes.byref(sch), arr, self.nblock,
                                        ctypes.byref(h)), "sg_create")
        self.h = h
        # three state buffers per block, one allocation each
        self.store = [torch.empty((3,) + s, dtype=dtype, device=device)
                      for s in self.shapes]
        for b, st in enumerate(self.store):
            _lib.check(self.L.sg_bind(self.h, b, st[0].data_ptr(),
                                      st[1].data_ptr(), st[2].data_ptr()),
                       "sg_bind")
        # the passive scalars' three buffers per block, rotated with the state
        self.sstore = []
        for b, d in enumerate(blocks):
            ns = int(d.get("nscalar", 0))
            t = None
            if ns:
                t = torch.zeros((3, ns) + self.shapes[b][1:], dtype=dtype,
                                device=device)
                _lib.check(self.L.sg_bind_scalars(self.h, b, t[0].data_ptr(),
                                                  t[1].data_ptr(), t[2].data_ptr()),
                           "sg_bind_scalars")
            self.sstore.append(t)
        # the FP64 scratch of the implicit solves (torch allocations)
        self.scratch = []
        for b in range(self.nblock):
            nb = ctypes.c_size_t()
            _lib.check(self.L.sg_scratch_bytes(self.h, b, ctypes.byref(nb)),
                       "sg_scratch_bytes")
            if nb.value:
                t = torch.empty(nb.value // 8, dtype=torch.float64, device=device)
                _lib.check(self.L.sg_bind_scratch(self.h, b, t.data_ptr(), nb.value),
                           "sg_bind_scratch")
                self.scratch.append(t)
        # the FluxRegister's step fields per block and direction, and the
        # implicit blocks' staging scratch for them (request_step_field)
        self.steps = [[None, None, None] for _ in range(self.nblock)]
        self.step_scratch = [None] * self.nblock
        self.dt = torch.zeros(self.nblock, dtype=torch.float64, device=device)
        self.redo = torch.zeros(self.nblock, dtype=torch.int32, device=device)
        self.flags = torch.zeros(self.nblock, dtype=torch.int32, device=device)
        # the device retry decision: 0 accepted, 1 redo, -1 terminated
        self.state = torch.zeros(self.nblock, dtype=torch.int32, device=device)
        self._w_ptrs = (ctypes.c_void_p * self.nblock)()

    def close(self) -> None:
        if getattr(self, "h", None):
            self.L.sg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- state ------------------------------------------------------------
    def current_index(self) -> int:
        c = ctypes.c_int32()
        _lib.check(self.L.sg_current(self.h, ctypes.byref(c)), "sg_current")
        return c.value

    def current(self, b: int = 0) -> torch.Tensor:
        return self.store[b][self.current_index()]

    def current_scalars(self, b: int = 0) -> Optional[torch.Tensor]:
        """Block b's current tracer densities (nscalar, nc3, nc2, nc1), or
        None without scalars."""
        t = self.sstore[b]
        return None if t is None else t[self.current_index()]

    def init_scalars(self, b: int, s: torch.Tensor, stream=None) -> None:
        """Block b's initial tracer densities into the current buffer, then
        their ghost cells by the boundary functions."""
        self.current_scalars(b).copy_(s)
        self.fill_ghosts(stream)

    def rotation(self):
        c, b = ctypes.c_int32(), ctypes.c_int32()
        _lib.check(self.L.sg_rotation(self.h, ctypes.byref(c), ctypes.byref(b)),
                   "sg_rotation")
        return c.value, b.value

    def set_rotation(self, rot) -> None:
        _lib.check(self.L.sg_set_rotation(self.h, rot[0], rot[1]), "sg_set_rotation")

    def advance(self, stage: int) -> None:
        _lib.check(self.L.sg_advance(self.h, stage), "sg_advance")

    def set_current(self, index: int) -> None:
        _lib.check(self.L.sg_set_current(self.h, index), "sg_set_current")

    def init_from_prim(self, ws: List[torch.Tensor], stream=None) -> None:
        for b, w in enumerate(ws):
            if w.dtype != torch.float64 or tuple(w.shape) != self.shapes[b]:
                raise ValueError(f"initialize: hydro_w of block {b} must be "
                                 f"float64 of shape {self.shapes[b]}, got "
                                 f"{w.dtype} {tuple(w.shape)}")
            if not w.is_contiguous() or w.device != self.device:
                raise ValueError("initialize: hydro_w must be contiguous on "
                                 f"{self.device}")
            self._w_ptrs[b] = w.data_ptr()
            if self.bases[b] is not None:
                self._set_base(b, w)
        self.set_current(0)
        _lib.check(self.L.sg_init_from_prim(self.h, self._w_ptrs, _stream(stream)),
                   "sg_init_from_prim")

    def _set_base(self, b: int, w: torch.Tensor) -> None:
        fill_base(self.bases[b], w, self.blocks[b])

    def totals(self, b: int, u: torch.Tensor) -> torch.Tensor:
        """The total conserved state (FP64) of block b's stored state u (an
        anomaly block adds its base)."""
        out = u.to(torch.float64)
        t = self.bases[b]
        if t is not None:
            nc1 = self.blocks[b]["nc1"]
            out[0] += t[0:nc1]
            out[4] += t[2 * nc1:3 * nc1]
        return out

    def prim(self, outs: List[torch.Tensor], stream=None) -> None:
        for b, w in enumerate(outs):
            if w.dtype != self.dtype or tuple(w.shape) != self.shapes[b]:
                raise ValueError("prim: output of the storage dtype and shape")
            self._w_ptrs[b] = w.data_ptr()
        _lib.check(self.L.sg_prim(self.h, self._w_ptrs, _stream(stream)), "sg_prim")

    # -- stepping -----------------------------------------------------------
    def stage(self, stage: int, stream=None, dt: Optional[torch.Tensor] = None) -> None:
        d = self.dt if dt is None else dt
        _lib.check(self.L.sg_stage(self.h, stage, d.data_ptr(), _stream(stream)),
                   "sg_stage")

    def max_dt(self, stream=None) -> torch.Tensor:
        """dt[b] = cfl 2^-redo[b] min(dx / (|v| + c)) on the device."""
        _lib.check(self.L.sg_max_dt(self.h, self.redo.data_ptr(), self.dt.data_ptr(),
                                    _stream(stream)), "sg_max_dt")
        return self.dt

    def check(self, stream=None) -> torch.Tensor:
        _lib.check(self.L.sg_check(self.h, self.flags.data_ptr(), _stream(stream)),
                   "sg_check")
        return self.flags

    def restore(self) -> None:
        _lib.check(self.L.sg_restore(self.h), "sg_restore")

    def check_retry(self, max_redo: int, stream=None) -> torch.Tensor:
        """After a step, on the device: the flags, and per block a redo
        (step-start state restored, redo += 1, state 1), a termination past
        max_redo (state -1, kept) or an accepted step (redo and state 0).
        The next max_dt halves the retried blocks' dt.  Returns the state."""
        _lib.check(self.L.sg_check_retry(self.h, self.flags.data_ptr(),
                                         self.redo.data_ptr(), int(max_redo),
                                         self.state.data_ptr(), _stream(stream)),
                   "sg_check_retry")
        return self.state

    def fill_ghosts(self, stream=None) -> None:
        _lib.check(self.L.sg_fill_ghosts(self.h, _stream(stream)), "sg_fill_ghosts")

    def tile(self, b: int = 0) -> int:
        t = ctypes.c_int32()
        _lib.check(self.L.sg_tile(self.h, b, ctypes.byref(t)), "sg_tile")
        return t.value

    def launches_per_stage(self) -> int:
        n = ctypes.c_int32()
        _lib.check(self.L.sg_launches_per_stage(self.h, ctypes.byref(n)),
                   "sg_launches_per_stage")
        return n.value

    def set_timing(self, on: bool) -> None:
        """Record device events around each kernel of every eager stage."""
        _lib.check(self.L.sg_set_timing(self.h, int(bool(on))), "sg_set_timing")

    def kernel_times(self) -> dict:
        """{kernel: (milliseconds, launches)} since the previous call (waits
        for the recorded events)."""
        n = len(_lib.KERNELS)
        ms = (ctypes.c_double * n)()
        cnt = (ctypes.c_int64 * n)()
        _lib.check(self.L.sg_kernel_times(self.h, ms, cnt), "sg_kernel_times")
        return {k: (ms[i], cnt[i]) for i, k in enumerate(_lib.KERNELS) if cnt[i]}

    # -- the FluxRegister's step fields and the budget sums ------------------
    def request_step_field(self, b: int, dim: int) -> torch.Tensor:
        """Allocate and bind the FP64 step field S_dim of block b
        (FluxRegister::request_step_field, src/hydro/flux_register.hpp:270):
        (5, nc3, nc2, nc1), zero, written by every stage from the next step
        on.  Returns the field."""
        if dim not in (1, 2, 3):
            raise ValueError(f"request_step_field: dim {dim}")
        nc = {1: self.blocks[b]["nc1"], 2: self.blocks[b]["nc2"],
              3: self.blocks[b]["nc3"]}[dim]
        if nc <= 1:
            raise ValueError(f"request_step_field: block {b} has no x{dim} faces")
        if self.steps[b][dim - 1] is None:
            self.steps[b][dim - 1] = torch.zeros(self.shapes[b], dtype=torch.float64,
                                                 device=self.device)
        self._bind_steps(b)
        return self.steps[b][dim - 1]

    def step_field(self, b: int, dim: int) -> Optional[torch.Tensor]:
        return self.steps[b][dim - 1]

    def _bind_steps(self, b: int) -> None:
        f = self.steps[b]
        nb = ctypes.c_size_t()
        _lib.check(self.L.sg_step_scratch_bytes(self.h, b, ctypes.byref(nb)),
                   "sg_step_scratch_bytes")
        if f[0] is not None and nb.value and self.step_scratch[b] is None:
            self.step_scratch[b] = torch.empty(nb.value // 8, dtype=torch.float64,
                                               device=self.device)
        t = self.step_scratch[b]
        ptr = [x.data_ptr() if x is not None else None for x in f]
        _lib.check(self.L.sg_bind_step_fields(
            self.h, b, ptr[0], ptr[1], ptr[2],
            t.data_ptr() if t is not None else None,
            t.numel() * 8 if t is not None else 0), "sg_bind_step_fields")

    def budget_totals(self, stream=None, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """(nblock, 5) FP64 on the device: each block's interior sum of the
        total conserved state times the cell volume."""
        if out is None:
            out = torch.empty((self.nblock, 5), dtype=torch.float64, device=self.device)
        _lib.check(self.L.sg_budget_totals(self.h, out.data_ptr(), _stream(stream)),
                   "sg_budget_totals")
        return out

    def budget_boundary(self, out: Optional[torch.Tensor] = None,
                        accumulate: bool = False, stream=None) -> torch.Tensor:
        """(nblock, 5) FP64 on the device: the outward transfer of the step
        fields through each block's boundary faces; accumulate adds it to
        out."""
        if out is None:
            out = torch.zeros((self.nblock, 5), dtype=torch.float64, device=self.device)
        _lib.check(self.L.sg_budget_boundary(self.h, out.data_ptr(), int(bool(accumulate)),
                                             _stream(stream)), "sg_budget_boundary")
        return out

    # -- the schedule autotuner ---------------------------------------------
    def autotune(self, reps: int = 3, use_cache: bool = True) -> dict:
        """Time the tile widths and the implicit finish forms on this
        batch's blocks and current state (or recall a cached choice) and
        apply the fastest; see ``snapy_gb300.autotune``."""
        from . import autotune as _at
        with torch.cuda.device(self.device):
            self.schedule = _at.tune(self, reps=reps, use_cache=use_cache)
        return self.schedule

    def solve_fallbacks(self) -> List[int]:
        """Per block, the columns the refined implicit solve has left to the
        direct FP64 solve so far (the reference's implicit.fp64_columns)."""
        out = (ctypes.c_int64 * self.nblock)()
        _lib.check(self.L.sg_solve_fallbacks(self.h, out), "sg_solve_fallbacks")
        return list(out)

    def set_sweep(self, mode: int) -> None:
        """The order of elimination of the scheme-9 solve of FP64-assembled
        blocks: 0 the serial sweep (the reference's order, bit for bit), 1
        the partitioned form (four chunks per column at once and a
        separator system; the same solution to rounding), 2 the autotuner's
        choice between them (serial until it runs)."""
        _lib.check(self.L.sg_set_sweep(self.h, int(mode)), "sg_set_sweep")
        self.sweep_mode = int(mode)

    def add_step_counts(self, acc: torch.Tensor, stream=None) -> torch.Tensor:
        """acc (nblock, 2) int64 on the device += the last step's monitor
        counts per block: riemann.pstar_clamp, implicit.fp64_columns."""
        if acc.dtype != torch.int64 or tuple(acc.shape) != (self.nblock, 2) \
                or not acc.is_contiguous() or acc.device != self.device:
            raise ValueError("add_step_counts: a contiguous (nblock, 2) int64 "
                             f"tensor on {self.device}")
        _lib.check(self.L.sg_add_step_counts(self.h, acc.data_ptr(), _stream(stream)),
                   "sg_add_step_counts")
        return acc

    def sweep(self) -> int:
        """1 while the partitioned form runs, else 0."""
        on = ctypes.c_int32()
        _lib.check(self.L.sg_sweep(self.h, ctypes.byref(on)), "sg_sweep")
        return on.value

    def set_solve(self, corrections: int) -> None:
        """The solve of implicit-precision float32 blocks: refined with that
        many FP64-residual corrections (1 to 3; 2 by default), 0 for the
        direct FP64 solve of every column, or -1 for the FP32 solve (the
        reference's FP32 compute: the sweep alone, the FP64 solve for the
        columns whose sweep fails)."""
        _lib.check(self.L.sg_set_solve(self.h, int(corrections)), "sg_set_solve")
