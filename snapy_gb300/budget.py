"""The conservation budget of a block from its FluxRegister step fields.

Mirrors ``BudgetConsumer`` (src/diagnostics/budget.hpp:37-90,
src/diagnostics/budget.cpp:68-260) -- which itself has no fixer, source or
residual columns yet (its O8-cols) -- with the monitor's counters and minima
and the restart carry: per block, in FP64,

* ``total``    the row totals of the conserved state over the interior (the
               base added back for an FP32 anomaly block) times the cell volume;
* ``change``   total minus the total at the interval's start;
* ``boundary`` the outward transfer through the block's boundary faces, the
               sum over the steps of the interval of sign A_f S_d on the wall
               and extrapolation faces (never periodic faces).

For the conserved rows without sources, ``change + boundary`` is zero to
roundoff.  Both sums run on the device (``sg_budget_totals``,
``sg_budget_boundary``) and read nothing back until ``flush``; an ``observe``
is two launches and may sit in a captured graph's stream order.

The monitor (RegisterMonitor, src/hydro/flux_register.hpp:61-178) has the
reference's counter names (src/hydro/hydro.cpp:175-192) and its one minimum,
summed over the accepted steps of the interval.  The device counts two of
them (``sg_add_step_counts``): ``riemann.pstar_clamp`` (interior HLLC faces
whose contact pressure was clamped to zero) and ``implicit.fp64_columns``
(columns the FP32 implicit solve left to its FP64 retry).  The others stay
zero on every deck this path accepts, as they would in the reference: the
face floors (``face_floor.*``) run only with ``eos.limiter``, which the deck
reader refuses; ``riemann.llf`` is the Euler Roe solver's, not built;
``thermo.*`` are the moist saturation adjustment's; nothing in the reference
writes the ``ef.*`` counters or the ``ef.pos_min`` minimum (+inf: unset).

``carry`` and ``resume`` are the restart carry of an interval still open
(BudgetCarry, src/output/restart.hpp:37-52): ``write_budget_carry`` /
``read_budget_carry`` put it in a restart part under ``budget_carry.*``.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np
import torch

ROWS = ["mass", "momentum1", "momentum2", "momentum3", "energy"]
# the register's counters and minima, in the reference's order
COUNTERS = ["ef.floor_patch", "ef.nan", "ef.vapor_fail", "ef.heat_capacity",
            "ef.pos_hits", "ef.pos_severe", "ef.scalar_pos_hits",
            "face_floor.rho", "face_floor.p", "face_floor.species",
            "riemann.pstar_clamp", "riemann.llf",
            "thermo.temp_solve", "thermo.pres_solve", "implicit.fp64_columns"]
MINIMA = ["ef.pos_min"]
# sg_add_step_counts' slot of each counter the device counts
DEVICE_SLOTS = {"riemann.pstar_clamp": 0, "implicit.fp64_columns": 1}
CARRY_PREFIX = "budget_carry."


@dataclass
class BudgetRecord:
    """One interval of the budget (BudgetRecord, budget.hpp:21-31)."""
    rows: List[str] = field(default_factory=lambda: list(ROWS))
    counters: List[str] = field(default_factory=lambda: list(COUNTERS))
    minima: List[str] = field(default_factory=lambda: list(MINIMA))
    total: Optional[np.ndarray] = None
    change: Optional[np.ndarray] = None
    boundary: Optional[np.ndarray] = None
    counter: Optional[np.ndarray] = None   # int64 per counter
    minimum: Optional[np.ndarray] = None   # FP64 per minimum, +inf: unset
    time: float = 0.0
    interval: float = 0.0
    dt: float = 0.0
    cycle: int = 0


@dataclass
class BudgetCarry:
    """An interval still open at a restart (BudgetCarry,
    src/output/restart.hpp:37-46): the sums since its start, on the host."""
    rows: List[str]
    total_prev: np.ndarray
    pending: np.ndarray
    counter: np.ndarray
    minimum: np.ndarray
    interval: float


def _pack_names(names: List[str]) -> torch.Tensor:
    """The names as one int8 tensor, newline-terminated (restart.cpp's
    pack_names)."""
    raw = "".join(n + "\n" for n in names).encode()
    return torch.tensor(list(raw), dtype=torch.uint8).view(torch.int8)


def _unpack_names(t: torch.Tensor) -> List[str]:
    raw = bytes(t.contiguous().view(torch.uint8).tolist()).decode()
    return [n for n in raw.split("\n")][:-1] if raw else []


def write_budget_carry(carry: Optional[BudgetCarry], out: dict) -> None:
    """write_budget_carry (src/output/restart.cpp:383-391): nothing for an
    undefined carry."""
    if carry is None:
        return
    out[CARRY_PREFIX + "rows"] = _pack_names(carry.rows)
    out[CARRY_PREFIX + "total_prev"] = torch.as_tensor(carry.total_prev, dtype=torch.float64)
    out[CARRY_PREFIX + "pending"] = torch.as_tensor(carry.pending, dtype=torch.float64)
    out[CARRY_PREFIX + "counter"] = torch.as_tensor(carry.counter, dtype=torch.int64)
    out[CARRY_PREFIX + "minimum"] = torch.as_tensor(carry.minimum, dtype=torch.float64)
    out[CARRY_PREFIX + "interval"] = torch.tensor([float(carry.interval)],
                                                  dtype=torch.float64)


def read_budget_carry(data: dict, rows: List[str]) -> Optional[BudgetCarry]:
    """read_budget_carry (src/output/restart.cpp:393-407): None when the
    file holds none or one with other rows (a new interval)."""
    keys = ("rows", "total_prev", "pending", "counter", "minimum", "interval")
    if any(CARRY_PREFIX + k not in data for k in keys):
        return None
    saved = _unpack_names(data[CARRY_PREFIX + "rows"])
    if saved != list(rows):
        return None
    return BudgetCarry(rows=saved,
                       total_prev=data[CARRY_PREFIX + "total_prev"].double().numpy(),
                       pending=data[CARRY_PREFIX + "pending"].double().numpy(),
                       counter=data[CARRY_PREFIX + "counter"].long().numpy(),
                       minimum=data[CARRY_PREFIX + "minimum"].double().numpy(),
                       interval=float(data[CARRY_PREFIX + "interval"].item()))


class BudgetConsumer:
    """The budget of one MeshBlock.  ``bind`` requests the step fields of the
    block's active directions (BudgetOutput::bind,
    src/output/budget_series.cpp:174-183); ``observe`` after every step
    adds the step's boundary transfer; ``flush`` closes the interval."""

    def __init__(self):
        self._started = False
        self._total_start: Optional[torch.Tensor] = None
        self._pending: Optional[torch.Tensor] = None
        self._counts: Optional[torch.Tensor] = None  # (1, 2) device slots
        self._counter0 = np.zeros(len(COUNTERS), dtype=np.int64)
        self._minimum = np.full(len(MINIMA), np.inf)
        self._interval = 0.0
        self._dt = 0.0
        self._cycle = 0
        self._local = BudgetRecord()

    @staticmethod
    def bind(block) -> None:
        c = block.options.coord()
        reg = block.flux_register()
        for d, n in ((1, c.nc1), (2, c.nc2), (3, c.nc3)):
            if n > 1:
                reg.request_step_field(d)

    @staticmethod
    def totals(block) -> torch.Tensor:
        """(5,) FP64 on the device: the interior totals of the current state."""
        with torch.cuda.device(block.device):
            return block.batch.budget_totals()[0]

    @staticmethod
    def boundary(block) -> torch.Tensor:
        """(5,) FP64 on the device: the outward transfer of the step fields
        of the last step through the boundary faces."""
        with torch.cuda.device(block.device):
            return block.batch.budget_boundary()[0]

    def _start(self, block) -> None:
        with torch.cuda.device(block.device):
            self._total_start = block.batch.budget_totals()
            self._pending = torch.zeros_like(self._total_start)
            self._counts = torch.zeros((block.batch.nblock, 2), dtype=torch.int64,
                                       device=block.device)
        self._counter0 = np.zeros(len(COUNTERS), dtype=np.int64)
        self._minimum = np.full(len(MINIMA), np.inf)
        self._interval = 0.0
        self._started = True

    def observe(self, block, vars: dict, dt: float) -> None:
        """After an accepted step: its boundary transfer and its monitor
        counts join the interval (the first observe starts the interval
        instead, its own step left out)."""
        self._dt = float(dt)
        self._cycle += 1
        if not self._started:
            self._start(block)
            return
        with torch.cuda.device(block.device):
            block.batch.budget_boundary(self._pending, accumulate=True)
            block.batch.add_step_counts(self._counts)
        self._interval += float(dt)

    def _counter(self) -> np.ndarray:
        """The interval's counters: the carried part and the device's."""
        c = self._counter0.copy()
        if self._counts is not None:
            dev = self._counts[0].cpu().numpy()
            for name, slot in DEVICE_SLOTS.items():
                c[COUNTERS.index(name)] += dev[slot]
        return c

    def flush(self, block, vars: dict, time: float) -> BudgetRecord:
        """Close the interval: the record, then a new interval from here."""
        if not self._started:
            self._start(block)
        with torch.cuda.device(block.device):
            total = block.batch.budget_totals()
        t = total[0].cpu().numpy()
        rec = BudgetRecord(total=t.copy(),
                           change=(total - self._total_start)[0].cpu().numpy(),
                           boundary=self._pending[0].cpu().numpy().copy(),
                           counter=self._counter(), minimum=self._minimum.copy(),
                           time=float(time), interval=self._interval,
                           dt=self._dt, cycle=self._cycle)
        self._local = rec
        self._total_start = total
        self._pending.zero_()
        self._counts.zero_()
        self._counter0[:] = 0
        self._minimum[:] = np.inf
        self._interval = 0.0
        return rec

    def carry(self, block, vars: dict, fires_now: bool = False) -> Optional[BudgetCarry]:
        """The sums since the interval's start, for a restart
        (BudgetConsumer::carry, src/diagnostics/budget.cpp:214-236); None
        before the interval started.  fires_now: the record at this time is
        still to come in the same output pass, so the carry starts a new
        interval from here."""
        if not self._started:
            return None
        if fires_now:
            with torch.cuda.device(block.device):
                total = block.batch.budget_totals()[0].cpu().numpy()
            return BudgetCarry(rows=list(ROWS), total_prev=total,
                               pending=np.zeros(len(ROWS)),
                               counter=np.zeros(len(COUNTERS), dtype=np.int64),
                               minimum=np.full(len(MINIMA), np.inf), interval=0.0)
        return BudgetCarry(rows=list(ROWS),
                           total_prev=self._total_start[0].cpu().numpy().copy(),
                           pending=self._pending[0].cpu().numpy().copy(),
                           counter=self._counter(), minimum=self._minimum.copy(),
                           interval=self._interval)

    def resume(self, block, carry: Optional[BudgetCarry]) -> None:
        """Resume the interval from a carry (BudgetConsumer::resume,
        src/diagnostics/budget.cpp:238-248); nothing for None."""
        if carry is None:
            return
        with torch.cuda.device(block.device):
            self._total_start = torch.as_tensor(
                carry.total_prev, dtype=torch.float64).view(1, -1).to(block.device)
            self._pending = torch.as_tensor(
                carry.pending, dtype=torch.float64).view(1, -1).to(block.device)
            self._counts = torch.zeros((block.batch.nblock, 2), dtype=torch.int64,
                                       device=block.device)
        self._counter0 = np.asarray(carry.counter, dtype=np.int64).copy()
        self._minimum = np.asarray(carry.minimum, dtype=np.float64).copy()
        self._interval = float(carry.interval)
        self._started = True

    def local(self) -> BudgetRecord:
        return self._local
