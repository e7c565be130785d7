"""The conservation budget of a block from its FluxRegister step fields.

Mirrors ``BudgetConsumer`` (src/diagnostics/budget.hpp:37-90,
src/diagnostics/budget.cpp:68-200) without the fixer, source and residual
columns, the monitor counters and the restart carry: per block, in FP64,

* ``total``    the row totals of the conserved state over the interior (the
               base added back for an FP32 anomaly block) times the cell volume;
* ``change``   total minus the total at the interval's start;
* ``boundary`` the outward transfer through the block's boundary faces, the
               sum over the steps of the interval of sign A_f S_d on the wall
               and extrapolation faces (never periodic faces).

For the conserved rows without sources, ``change + boundary`` is zero to
roundoff.  Both sums run on the device (``sg_budget_totals``,
``sg_budget_boundary``) and read nothing back until ``flush``; an ``observe``
is one launch and may sit in a captured graph's stream order.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np
import torch

ROWS = ["mass", "momentum1", "momentum2", "momentum3", "energy"]


@dataclass
class BudgetRecord:
    """One interval of the budget (BudgetRecord, budget.hpp:21-31)."""
    rows: List[str] = field(default_factory=lambda: list(ROWS))
    total: Optional[np.ndarray] = None
    change: Optional[np.ndarray] = None
    boundary: Optional[np.ndarray] = None
    time: float = 0.0
    interval: float = 0.0
    dt: float = 0.0
    cycle: int = 0


class BudgetConsumer:
    """The budget of one MeshBlock.  ``bind`` requests the step fields of the
    block's active directions (BudgetOutput::bind,
    src/output/budget_series.cpp:174-183); ``observe`` after every step
    adds the step's boundary transfer; ``flush`` closes the interval."""

    def __init__(self):
        self._started = False
        self._total_start: Optional[torch.Tensor] = None
        self._pending: Optional[torch.Tensor] = None
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
        self._interval = 0.0
        self._started = True

    def observe(self, block, vars: dict, dt: float) -> None:
        """After a step: its boundary transfer joins the interval (the first
        observe starts the interval instead, its own step left out)."""
        self._dt = float(dt)
        self._cycle += 1
        if not self._started:
            self._start(block)
            return
        with torch.cuda.device(block.device):
            block.batch.budget_boundary(self._pending, accumulate=True)
        self._interval += float(dt)

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
                           time=float(time), interval=self._interval,
                           dt=self._dt, cycle=self._cycle)
        self._local = rec
        self._total_start = total
        self._pending.zero_()
        self._interval = 0.0
        return rec

    def local(self) -> BudgetRecord:
        return self._local
