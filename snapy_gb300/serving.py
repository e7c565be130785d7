"""Serving: hydro solves of different sizes, admitted as they arrive and
advanced together on one GPU (continuous batching).

A request is a deck (its own grid), a seeded initial state and a number of
RK3 steps.  The server admits arrived requests first come, first served, as
long as their device memory fits the HBM budget (by default the free memory
the device reports, less a reserve).  An admitted request owns its device
state -- three state buffers, the implicit solve's and x3 sweep's scratch,
the FP32 hydrostatic base and its x1 geometry -- for its whole life.

Every running request advances in the SAME launches: the running set is one
library handle (a batch of blocks of uneven size), one step = each block's
own CFL time step on the device, then the three stages.  When the running
set changes (an admission or a completion) the handle is rebuilt over the
requests' existing buffers: each request's buffers are bound in the order
that puts its current state at the handle's current index, so requests that
joined at different steps share one buffer rotation.  Each block's result
depends on its own data only (tiles and columns never mix blocks), so a
request's result is bit for bit the same alone and in any mix.

Finished requests copy their state to pinned host memory asynchronously;
the host loop stays at most two steps ahead of the GPU, so completion times
are seen within a step.  Latency = result on the host - arrival.

The reference serves nothing of this kind; its Mesh advances a fixed set of
equal blocks on worker threads (src/mesh/mesh.cpp:374-410).
"""
from __future__ import annotations

import collections
import ctypes
import time
from dataclasses import dataclass
from typing import Callable, List, Optional

import torch

from . import _lib
from .batch import _DT, _stream, fill_base
from .meshblock import block_of, scheme_of
from .options import DeckError, MeshBlockOptions, shared_solve, shared_sweep


@dataclass
class Request:
    rid: int
    options: MeshBlockOptions
    initial: Callable[[], torch.Tensor]  # -> FP64 hydro_w of the deck's shape
    steps: int
    arrival: float = 0.0  # seconds after the server starts
    admitted: Optional[float] = None
    done: Optional[float] = None
    result: Optional[torch.Tensor] = None  # the final stored state (host)
    flags: int = 0
    # a deck with passive scalars: -> FP64 scalar_r (nscalar, nc3, nc2, nc1)
    tracers: Optional[Callable[[], torch.Tensor]] = None
    result_scalars: Optional[torch.Tensor] = None  # the final scalar_s (host)

    @property
    def latency(self) -> Optional[float]:
        return None if self.done is None else self.done - self.arrival

    @property
    def cells(self) -> int:
        c = self.options.coord()
        return c.nx1 * c.nx2 * c.nx3


def footprint(options: MeshBlockOptions, dtype: torch.dtype) -> int:
    """Device bytes a request holds while admitted."""
    c = options.coord()
    h = options.hydro()
    s = torch.finfo(dtype).bits // 8
    nc = c.nc1 * c.nc2 * c.nc3
    icells = c.nx1 * c.nx2 * c.nx3
    b = 3 * 5 * nc * s
    if h.icorr is not None:
        b += icells * 100 * 8
        if h.precision == "float32" and h.icorr.precision == "float32":
            # the refined solve's FP32 part
            b += (icells * 160 + (icells // c.nx1) * 7) * 4 + 16
    if c.nx3 > 1:
        b += 5 * icells * s
    ns = len(options.scalar_names)
    if ns:  # the tracers' buffers and their face scratch
        b += 3 * ns * nc * s + (4 + 5 * ns) * nc * 8
    b += 8 * (5 * c.nc1 + 1) + 16 * (c.nc1 + 1)
    return b


class _Slot:
    """An admitted request's device state, bound into every handle it runs
    in."""

    def __init__(self, req: Request, device, dtype):
        self.ns = len(req.options.scalar_names)
        if self.ns and req.tracers is None:
            raise DeckError(f"request {req.rid}: its deck carries passive "
                            "scalars; the request needs their scalar_r (tracers)")
        self.req = req
        self.desc = d = block_of(req.options)
        self.shape = (5, d["nc3"], d["nc2"], d["nc1"])
        self.store = torch.empty((3,) + self.shape, dtype=dtype, device=device)
        self.sstore = (torch.empty((3, self.ns) + self.shape[1:], dtype=dtype,
                                   device=device) if self.ns else None)
        self.x1f = torch.as_tensor(d["x1f"], dtype=torch.float64, device=device)
        self.x1v = torch.as_tensor(d["x1v"], dtype=torch.float64, device=device)
        self.base = None
        if dtype == torch.float32 and d.get("grav1", 0.0) != 0.0:
            self.base = torch.zeros(5 * d["nc1"] + 1, dtype=torch.float64,
                                    device=device)
        self.scratch = None
        self.cur = 0
        self.perm = (0, 1, 2)
        self.step = 0
        self.bytes = footprint(req.options, dtype)


def _descs(slots: List[_Slot]):
    arr = (_lib.BlockDesc * len(slots))()
    for b, sl in enumerate(slots):
        a, d = arr[b], sl.desc
        a.nc1, a.nc2, a.nc3, a.ng = d["nc1"], d["nc2"], d["nc3"], d["ng"]
        for f in range(6):
            a.bc[f] = d["bc"][f]
        a.dx1, a.dx2, a.dx3 = d["dx1"], d["dx2"], d["dx3"]
        a.gammad = d["gammad"]
        a.tj = 0
        a.grav1 = d.get("grav1", 0.0)
        a.nu_iso = d.get("nu_iso", 0.0)
        a.flux_cov = int(bool(d.get("flux_cov", True)))
        a.wb_wall_clamp = int(bool(d.get("wb_wall_clamp", True)))
        a.x1f = sl.x1f.data_ptr()
        a.x1v = sl.x1v.data_ptr()
        a.implicit_scheme = int(d.get("implicit_scheme", 0))
        a.implicit_precision = _lib.F32 if d.get("implicit_f32") else _lib.F64
        a.base = sl.base.data_ptr() if sl.base is not None else None
        a.nscalar = int(d.get("nscalar", 0))
    return arr


class _Handle:
    """One library handle over the running slots' buffers."""

    def __init__(self, L, sch, slots: List[_Slot], device):
        self.L = L
        self.slots = list(slots)
        n = len(slots)
        h = ctypes.c_void_p()
        _lib.check(L.sg_create(ctypes.byref(sch), _descs(slots), n,
                               ctypes.byref(h)), "sg_create")
        self.h = h
        for b, sl in enumerate(slots):
            # the slot's current state at handle index 0
            sl.perm = (sl.cur, (sl.cur + 1) % 3, (sl.cur + 2) % 3)
            _lib.check(L.sg_bind(h, b, *(sl.store[q].data_ptr() for q in sl.perm)),
                       "sg_bind")
            if sl.sstore is not None:
                _lib.check(L.sg_bind_scalars(
                    h, b, *(sl.sstore[q].data_ptr() for q in sl.perm)),
                    "sg_bind_scalars")
            nb = ctypes.c_size_t()
            _lib.check(L.sg_scratch_bytes(h, b, ctypes.byref(nb)), "sg_scratch_bytes")
            if nb.value:
                if sl.scratch is None or sl.scratch.numel() * 8 < nb.value:
                    sl.scratch = torch.empty((nb.value + 7) // 8, dtype=torch.float64,
                                             device=device)
                _lib.check(L.sg_bind_scratch(h, b, sl.scratch.data_ptr(),
                                             sl.scratch.numel() * 8),
                           "sg_bind_scratch")
        _lib.check(L.sg_set_current(h, 0), "sg_set_current")
        k = shared_solve(sl.req.options.solve_corrections() for sl in slots)
        if k != 2:
            _lib.check(L.sg_set_solve(h, k), "sg_set_solve")
        # the partitioned sweep when every request asks for it (a served
        # handle runs no autotuner, so "auto" keeps the serial sweep)
        if shared_sweep(sl.req.options.sweep_mode() for sl in slots) == 1:
            _lib.check(L.sg_set_sweep(h, 1), "sg_set_sweep")
        self.dt = torch.zeros(n, dtype=torch.float64, device=device)
        self.redo = torch.zeros(n, dtype=torch.int32, device=device)
        self.flags = torch.zeros(n, dtype=torch.int32, device=device)

    def step(self, nstage: int, stream) -> None:
        s = _stream(stream)
        _lib.check(self.L.sg_max_dt(self.h, self.redo.data_ptr(), self.dt.data_ptr(), s),
                   "sg_max_dt")
        for st in range(nstage):
            _lib.check(self.L.sg_stage(self.h, st, self.dt.data_ptr(), s), "sg_stage")

    def current(self) -> int:
        c, b = ctypes.c_int32(), ctypes.c_int32()
        _lib.check(self.L.sg_rotation(self.h, ctypes.byref(c), ctypes.byref(b)),
                   "sg_rotation")
        return c.value

    def check(self, stream) -> torch.Tensor:
        _lib.check(self.L.sg_check(self.h, self.flags.data_ptr(), _stream(stream)),
                   "sg_check")
        return self.flags

    def launches_per_step(self, nstage: int) -> int:
        n = ctypes.c_int32()
        _lib.check(self.L.sg_launches_per_stage(self.h, ctypes.byref(n)),
                   "sg_launches_per_stage")
        return 2 + nstage * n.value

    def close(self) -> None:
        if self.h:
            self.L.sg_destroy(self.h)
            self.h = None


class Server:
    """Continuous batching of hydro solves on one device.

    All requests must share one scheme (solver, reconstruction, RK weights,
    CFL, floors) and one storage precision; their grids may differ."""

    def __init__(self, device: Optional[torch.device] = None,
                 hbm_budget: Optional[int] = None, reserve: int = 2 << 30,
                 timing: bool = False):
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        self.hbm_budget = hbm_budget
        self.reserve = reserve
        self.L = _lib.load()
        self.max_running = 0
        self.rebuilds = 0
        self.budget: Optional[int] = None  # the budget of the last run
        self.gpu_step_ms: List[float] = []
        self.launches = 0
        self.h2d_bytes = 0
        self.d2h_bytes = 0
        # per-kernel device time of every step (sg_set_timing), when asked
        self.timing = timing
        self.kernel_ms = {}

    def _close(self, handle) -> None:
        if self.timing:
            n = len(_lib.KERNELS)
            ms = (ctypes.c_double * n)()
            cnt = (ctypes.c_int64 * n)()
            _lib.check(self.L.sg_kernel_times(handle.h, ms, cnt), "sg_kernel_times")
            for i, k in enumerate(_lib.KERNELS):
                if cnt[i]:
                    a = self.kernel_ms.setdefault(k, [0.0, 0])
                    a[0] += ms[i]
                    a[1] += cnt[i]
        handle.close()

    def _scheme(self, requests: List[Request]):
        schemes = [scheme_of(r.options) for r in requests]
        if any(s != schemes[0] for s in schemes[1:]):
            raise DeckError("served requests must share one scheme")
        prec = {r.options.hydro().precision for r in requests}
        if len(prec) != 1:
            raise DeckError("served requests must share dynamics/precision")
        dtype = torch.float64 if prec.pop() == "float64" else torch.float32
        sc = schemes[0]
        sch = _lib.Scheme()
        sch.dtype = _DT[dtype]
        sch.riemann = sc["riemann"]
        sch.shock = int(sc["shock"])
        sch.scale = int(sc["scale"])
        sch.nstage = len(sc["wght"])
        for s, w in enumerate(sc["wght"]):
            for q in range(3):
                sch.wght[s][q] = w[q]
        sch.cfl = sc["cfl"]
        sch.density_floor = sc["density_floor"]
        sch.pressure_floor = sc["pressure_floor"]
        return sch, dtype, len(sc["wght"])

    def _admit(self, req: Request, sch, dtype, stream) -> _Slot:
        sl = _Slot(req, self.device, dtype)
        w = req.initial()
        w = w.to(self.device, torch.float64, non_blocking=True).contiguous()
        self.h2d_bytes += w.numel() * 8
        if sl.base is not None:
            fill_base(sl.base, w, sl.desc)
        tmp = _Handle(self.L, sch, [sl], self.device)
        try:
            ptrs = (ctypes.c_void_p * 1)(w.data_ptr())
            _lib.check(self.L.sg_init_from_prim(tmp.h, ptrs, _stream(stream)),
                       "sg_init_from_prim")
            if sl.ns:
                # scalar_s = rho scalar_r from the FP64 initial density, as
                # MeshBlock.initialize sets it, then its ghosts
                r = req.tracers().to(self.device, torch.float64)
                self.h2d_bytes += r.numel() * 8
                sl.sstore[0].copy_((w[0].unsqueeze(0) * r).to(dtype))
                _lib.check(self.L.sg_fill_ghosts(tmp.h, _stream(stream)),
                           "sg_fill_ghosts")
        finally:
            tmp.close()
        sl.cur = 0
        return sl

    def run(self, requests: List[Request]) -> List[Request]:
        """Serve `requests` (their arrival times are seconds after the call)
        to completion; fills admitted / done / result / flags of each."""
        if not requests:
            return requests
        sch, dtype, nstage = self._scheme(requests)
        with torch.cuda.device(self.device):
            stream = torch.cuda.current_stream()
            budget = self.hbm_budget
            if budget is None:
                free, _ = torch.cuda.mem_get_info(self.device)
                budget = max(0, free - self.reserve)
            self.budget = budget
            pending = sorted(requests, key=lambda r: (r.arrival, r.rid))
            running: List[_Slot] = []
            finishing = []
            inflight = collections.deque()
            handle: Optional[_Handle] = None
            dirty = True
            used = 0
            t0 = time.perf_counter()
            while pending or running or finishing:
                now = time.perf_counter() - t0
                for item in list(finishing):
                    req, ev, host, flags = item
                    if ev.query():
                        req.done = time.perf_counter() - t0
                        req.result = host[0] if isinstance(host, tuple) else host
                        if isinstance(host, tuple):
                            req.result_scalars = host[1]
                        req.flags = int(flags.item())
                        finishing.remove(item)
                # first come, first served, while the memory fits
                while pending and pending[0].arrival <= now:
                    fp = footprint(pending[0].options, dtype)
                    if fp > budget:
                        raise RuntimeError(f"request {pending[0].rid} needs {fp} "
                                           f"device bytes, over the budget {budget}")
                    if used + fp > budget:
                        break
                    req = pending.pop(0)
                    req.admitted = time.perf_counter() - t0
                    running.append(self._admit(req, sch, dtype, stream))
                    used += fp
                    dirty = True
                if not running:
                    if pending and not finishing:
                        time.sleep(max(0.0, min(1e-3, pending[0].arrival - now)))
                    elif finishing:
                        finishing[0][1].synchronize()
                    continue
                if dirty:
                    if handle is not None:
                        self._close(handle)
                    handle = _Handle(self.L, sch, running, self.device)
                    if self.timing:
                        _lib.check(self.L.sg_set_timing(handle.h, 1), "sg_set_timing")
                    self.rebuilds += 1
                    dirty = False
                self.max_running = max(self.max_running, len(running))
                while len(inflight) >= 2:
                    inflight.popleft().synchronize()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                handle.step(nstage, stream)
                e1.record(stream)
                inflight.append(e1)
                self.gpu_step_ms.append((e0, e1))
                self.launches += handle.launches_per_step(nstage)
                c = handle.current()
                done_now = []
                for sl in running:
                    sl.cur = sl.perm[c]
                    sl.step += 1
                    if sl.step >= sl.req.steps:
                        done_now.append(sl)
                if done_now:
                    flags = handle.check(stream)
                    for sl in done_now:
                        b = running.index(sl)
                        host = torch.empty(sl.shape, dtype=dtype, pin_memory=True)
                        host.copy_(sl.store[sl.cur], non_blocking=True)
                        if sl.sstore is not None:
                            sh = torch.empty(sl.sstore.shape[1:], dtype=dtype,
                                             pin_memory=True)
                            sh.copy_(sl.sstore[sl.cur], non_blocking=True)
                            self.d2h_bytes += sh.numel() * sh.element_size()
                            host = (host, sh)
                        fh = torch.empty((), dtype=torch.int32, pin_memory=True)
                        fh.copy_(flags[b], non_blocking=True)
                        ev = torch.cuda.Event()
                        ev.record(stream)
                        finishing.append((sl.req, ev, host, fh))
                        hh = host[0] if isinstance(host, tuple) else host
                        self.d2h_bytes += hh.numel() * hh.element_size()
                    for sl in done_now:
                        running.remove(sl)
                        used -= sl.bytes
                    dirty = True
            if handle is not None:
                self._close(handle)
            torch.cuda.synchronize(self.device)
            self.gpu_step_ms = [a.elapsed_time(b) for a, b in self.gpu_step_ms]
        return requests
