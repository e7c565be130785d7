"""Batched ensembles: many blocks of one scheme advanced together on one GPU.

An ``Ensemble`` holds members of uneven size (each its own deck geometry and
initial state) in ONE library handle: every RK stage of every member is one
persistent launch of the stage kernel (plus the implicit solve's and the
ghost fill's), each member with its own time step computed on the device, and
a whole step -- time steps, three stages -- is captured once as a CUDA graph
and replayed.  There is no host synchronisation inside a step.

The reference advances equal-shape blocks one after another on worker
threads (src/mesh/mesh.cpp:374-410, one CUDA stream per block); members here
may differ in size and share the launch instead.
"""
from __future__ import annotations

from typing import List, Optional, Sequence

import torch

from .batch import Batch
from .meshblock import block_of, scheme_of
from .options import DeckError, MeshBlockOptions, shared_solve, shared_sweep


class Ensemble:
    def __init__(self, members: Sequence[MeshBlockOptions],
                 device: Optional[torch.device] = None,
                 dtype: Optional[torch.dtype] = None, graphs: bool = True,
                 retry: bool = False):
        if not members:
            raise ValueError("an ensemble needs at least one member")
        self.members = list(members)
        schemes = [scheme_of(m) for m in self.members]
        if any(s != schemes[0] for s in schemes[1:]):
            raise DeckError("ensemble members must share one scheme (solver, "
                            "reconstruction, RK weights, cfl, floors)")
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        prec = {m.hydro().precision for m in self.members}
        if dtype is None:
            if len(prec) != 1:
                raise DeckError("ensemble members must share dynamics/precision")
            dtype = torch.float64 if prec.pop() == "float64" else torch.float32
        self.dtype = dtype
        self.batch = Batch(schemes[0], [block_of(m) for m in self.members],
                           self.device, dtype)
        k = shared_solve(m.solve_corrections() for m in self.members)
        if k != 2:
            self.batch.set_solve(k)
        sw = shared_sweep(m.sweep_mode() for m in self.members)
        if sw:
            self.batch.set_sweep(sw)
        self.nstage = len(schemes[0]["wght"])
        self.graphs = graphs
        # retry on the device (MeshBlockImpl::apply_redo per member): each
        # step ends with the check, a rejected member gets its step-start
        # state back and its next dt halved, all inside the captured step
        self.retry = retry
        self.max_redo = self.members[0].intg().max_redo
        self._graphs = {}
        self._seen = set()
        self.replays = 0
        self.captures = 0
        self.time = torch.zeros(len(self.members), dtype=torch.float64,
                                device=self.device)

    def __len__(self):
        return len(self.members)

    @property
    def cells(self) -> int:
        n = 0
        for m in self.members:
            c = m.coord()
            n += c.nx1 * c.nx2 * c.nx3
        return n

    def initialize(self, ws: List[torch.Tensor], autotune: Optional[bool] = None,
                   rs: Optional[List[Optional[torch.Tensor]]] = None) -> None:
        """The members' initial primitives (and, for members with passive
        scalars, their ratios rs[k], scalar_s = rho r as MeshBlock.initialize
        sets it); then (autotune None: as the first member's
        integration/autotune) the schedule autotuner on the batch."""
        ws = [w.to(self.device, torch.float64).contiguous() for w in ws]
        with torch.cuda.device(self.device):
            self.batch.init_from_prim(ws)
            if self.members[0].autotune if autotune is None else autotune:
                self.batch.autotune()
                self._graphs.clear()
                self._seen.clear()
            if any(m.scalar_names for m in self.members):
                for k, m in enumerate(self.members):
                    if not m.scalar_names:
                        continue
                    r = rs[k] if rs is not None else None
                    if r is None:
                        raise RuntimeError(f"initialize: member {k} needs its "
                                           "scalar_r")
                    s = ws[k][0].unsqueeze(0) * r.to(self.device, torch.float64)
                    self.batch.current_scalars(k).copy_(s.to(self.dtype))
                self.batch.fill_ghosts()
        self.time.zero_()

    def scalars(self, k: int) -> Optional[torch.Tensor]:
        """Member k's current tracer densities (a view of block storage), or
        None without scalars."""
        return self.batch.current_scalars(k)

    def state(self, k: int) -> torch.Tensor:
        """The current conserved state of member k (a view of block storage)."""
        return self.batch.current(k)

    def max_time_step(self) -> torch.Tensor:
        with torch.cuda.device(self.device):
            return self.batch.max_dt()

    def _launch_step(self, fixed_dt: Optional[torch.Tensor]) -> None:
        b = self.batch
        if fixed_dt is None:
            b.max_dt()
        else:
            b.dt.copy_(fixed_dt)
        for s in range(self.nstage):
            b.stage(s)
        if self.retry:
            state = b.check_retry(self.max_redo)
            self.time.add_(torch.where(state == 0, b.dt, torch.zeros_like(b.dt)))
        else:
            self.time.add_(b.dt)

    def step(self, dt: Optional[torch.Tensor] = None) -> None:
        """One RK step of every member: each member's own CFL time step from
        the device (or the given per-member dt), all stages, as one graph."""
        with torch.cuda.device(self.device):
            b = self.batch
            rot = b.rotation()
            key = (rot, dt is None)
            g = self._graphs.get(key) if self.graphs else None
            if g is None and self.graphs and key in self._seen:
                g = torch.cuda.CUDAGraph()
                s = torch.cuda.Stream(device=self.device)
                s.wait_stream(torch.cuda.current_stream())
                self._fixed = torch.zeros_like(b.dt) if dt is not None else None
                try:
                    with torch.cuda.stream(s):
                        g.capture_begin()
                        try:
                            self._launch_step(self._fixed if dt is not None else None)
                        finally:
                            g.capture_end()
                finally:
                    b.set_rotation(rot)
                torch.cuda.current_stream().wait_stream(s)
                self._graphs[key] = (g, self._fixed)
                self.captures += 1
            if g is not None:
                graph, fixed = g if isinstance(g, tuple) else (g, None)
                if dt is not None:
                    fixed.copy_(dt)
                graph.replay()
                for st in range(self.nstage):
                    b.advance(st)
                self.replays += 1
            else:
                self._launch_step(dt)
                self._seen.add(key)

    @property
    def redo(self) -> torch.Tensor:
        """Per-member redo counts (device; retry mode)."""
        return self.batch.redo

    @property
    def outcome(self) -> torch.Tensor:
        """Per-member outcome of the last step (device; retry mode): 0
        accepted, 1 rejected and restored, -1 terminated."""
        return self.batch.state

    def check(self) -> torch.Tensor:
        """Per-member retry flags (one host read)."""
        with torch.cuda.device(self.device):
            return self.batch.check().cpu()
