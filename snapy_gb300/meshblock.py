"""``MeshBlock``: the reference's block API over the GB300 hydro stage.

Mirrors ``snapy.MeshBlock`` (python/csrc/pymesh.cpp:143-330 in the
reference): ``to``, ``initialize``, ``max_time_step``, ``forward(vars, dt,
stage)``, ``check_redo``, ``execution_report``, ``execution_capability``,
``part``, ``total_u``, ``intg``.  The stage itself runs in
``libsnapy_gb300.so``; this module only keeps the reference's bookkeeping
(variables dict, redo counter, graph cache).

State handling follows the reference's StateStore (src/mesh/state_store.hpp):
``vars["hydro_u"]`` is a view of block-owned storage; after every ``forward``
it is re-pointed (``Tensor.set_``) at the buffer holding the new state, so a
caller holding the tensor always sees the current state, and a tensor the
caller rebinds is adopted (copied in) at the next stage.
"""
from __future__ import annotations

import os

from dataclasses import dataclass
from typing import Dict, Optional

import torch

from . import _lib
from .batch import Batch
from .options import DeckError, MeshBlockOptions

kIDN, kIVX, kIVY, kIVZ, kIPR, kICY = 0, 1, 2, 3, 4, 5
kIV1 = kIVX

_BC = {"reflecting": _lib.BC_REFLECTING, "periodic": _lib.BC_PERIODIC,
       "extrapolation": _lib.BC_EXTRAPOLATION, "": _lib.BC_NONE,
       "custom": _lib.BC_NONE}


def scheme_of(options: MeshBlockOptions) -> dict:
    """The library scheme of a deck; refuses what the stage does not build."""
    h = options.hydro()
    c = options.coord()
    if c.type != "cartesian":
        raise DeckError(f"geometry/type '{c.type}': this stage builds cartesian")
    if h.eos.type != "ideal-gas":
        raise DeckError(f"equation-of-state '{h.eos.type}': this stage builds "
                        "ideal-gas")
    if h.eos.limiter:
        raise DeckError("equation-of-state/limiter: true is not built")
    if c.nghost != 3:
        raise DeckError(f"nghost {c.nghost}: weno5 needs nghost 3")
    for r in (h.recon1, h.recon23):
        if r.type != "weno5":
            raise DeckError(f"reconstruct type '{r.type}': weno5 is built")
    if (h.recon1.shock, h.recon1.scale) != (h.recon23.shock, h.recon23.scale):
        raise DeckError("vertical and horizontal reconstruct must share shock "
                        "and scale")
    if h.riemann.type not in ("hllc", "lmars"):
        raise DeckError(f"riemann-solver '{h.riemann.type}' is not built")
    if h.grav is not None:
        if h.grav.grav2 or h.grav.grav3:
            raise DeckError("forcing/const-gravity: grav2/grav3 are not built")
        if h.grav.non_hydrostatic != 1.0:
            raise DeckError("forcing/const-gravity/non-hydrostatic < 1 is not built")
        if h.grav.grav1 and h.precision == "float32" and h.riemann.type != "lmars":
            raise DeckError("dynamics/precision float32 under gravity is built "
                            "for the lmars solver (its state is stored as "
                            "anomalies about an FP64 hydrostatic base)")
    if h.diffusion is not None:
        extra = set(h.diffusion.raw) - {"nu_iso", "nu-iso"}
        if extra:
            raise DeckError(f"forcing/diffusion: {sorted(extra)} are not built "
                            "(nu_iso only)")
    if h.icorr is not None:
        if h.icorr.scheme not in (1, 9):
            raise DeckError(f"integration/implicit-scheme {h.icorr.scheme}: the "
                            "full 5x5 scheme 9 and the partial 3x3 scheme 1 "
                            "are built")
        if options.hydro().precision == "float64" and h.icorr.precision == "float32":
            raise DeckError("integration/implicit-precision float32 needs "
                            "dynamics/precision float32")
    intg = options.intg()
    return {
        "riemann": _lib.HLLC if h.riemann.type == "hllc" else _lib.LMARS,
        "shock": h.recon1.shock,
        "scale": h.recon1.scale,
        "wght": [(w.wght0, w.wght1, w.wght2) for w in intg.stages],
        "cfl": intg.cfl,
        "density_floor": h.eos.density_floor,
        "pressure_floor": h.eos.pressure_floor,
    }


def block_of(options: MeshBlockOptions, tj: int = 0) -> dict:
    c = options.coord()
    names = list(options.bcnames) + [""] * (6 - len(options.bcnames))
    bc = []
    for n in names[:6]:
        kind = n.rsplit("_", 1)[0] if n else ""
        if kind == "outflow":
            raise DeckError("boundary 'outflow' (radiating) is not built; "
                            "use extrapolation")
        if kind not in _BC:
            raise DeckError(f"boundary '{kind}' is not built")
        bc.append(_BC[kind])
    h = options.hydro()
    x1f = c.faces(1)
    x1v = 0.5 * (x1f[:-1] + x1f[1:])  # CoordinateImpl::x1_metrics_
    return {"nc1": c.nc1, "nc2": c.nc2, "nc3": c.nc3, "ng": c.nghost,
            "dx1": c.dx1, "dx2": c.dx2 if c.nx2 > 1 else (c.x2max - c.x2min),
            "dx3": c.dx3 if c.nx3 > 1 else (c.x3max - c.x3min),
            "gammad": h.eos.gammad, "bc": bc, "tj": tj,
            "grav1": h.grav.grav1 if h.grav else 0.0,
            "nu_iso": h.diffusion.nu_iso if h.diffusion else 0.0,
            "flux_cov": h.flux_covariance,
            "wb_wall_clamp": bool(h.extra.get("wb-wall-clamp", True)),
            "x1f": x1f, "x1v": x1v,
            "implicit_scheme": h.icorr.scheme if h.icorr else 0,
            # FP32 assembly of the implicit blocks (the solve is refined to,
            # or is, the FP64 solve: sg_set_solve)
            "implicit_f32": bool(h.icorr) and h.icorr.precision == "float32",
            "nscalar": len(options.scalar_names)}


class FluxRegister:
    """The step fields of a block's FluxRegister
    (src/hydro/flux_register.hpp:241-402): S_d <- w1 S_d + w2 dt T_d after
    every stage, in FP64, over the stage's face-flux totals T_d (the Riemann
    flux, the diffusion energy row, the prescribed walls and the implicit
    solve's x1 posts).  The totals themselves are not kept: the stage kernel
    folds them into S_d where it makes them."""

    def __init__(self, block: "MeshBlock"):
        self._blk = block

    def _active(self, dim: int) -> bool:
        c = self._blk.options.coord()
        return {1: c.nc1, 2: c.nc2, 3: c.nc3}.get(dim, 1) > 1

    def request_step_field(self, dim: int) -> None:
        """A reader asks for S_dim; it holds the step's sum from the next
        step on (request_step_field, flux_register.hpp:270)."""
        if not self._active(dim):
            raise RuntimeError(f"[FluxRegister] request_step_field: direction "
                               f"{dim} has no faces in this block")
        self._blk._step_dims.add(dim)
        if self._blk._batch is not None:
            with torch.cuda.device(self._blk.device):
                self._blk._batch.request_step_field(0, dim)

    def has_step_field(self, dim: int) -> bool:
        return dim in self._blk._step_dims

    def step_field(self, dim: int) -> torch.Tensor:
        """S_dim, (5, nc3, nc2, nc1) FP64 on the block's device; the faces of
        the interior cells are written, the rest stay zero."""
        if dim not in self._blk._step_dims:
            raise RuntimeError(f"[FluxRegister] step_field({dim}) was not "
                               "requested")
        return self._blk.batch.step_field(0, dim)


@dataclass
class _Intg:
    options: object
    current_redo: int = 0

    @property
    def stages(self):
        return self.options.stages


class _BlockModule:
    """A submodule view of a MeshBlock for module(name).buffer(name)."""

    BUFFERS = {
        "": ("hydro_u", "u0", "scalar_s", "x1f", "x1v", "x2f", "x2v", "x3f",
             "x3v", "hydro_ref"),
        "hydro": ("hydro_u", "u0", "hydro_ref"),
        "coord": ("x1f", "x1v", "x2f", "x2v", "x3f", "x3v"),
    }

    def __init__(self, block: "MeshBlock", name: str):
        self.block, self.name = block, name

    @property
    def options(self):
        o = self.block.options
        return {"": o, "hydro": o.hydro(), "coord": o.coord()}[self.name]

    def buffer(self, name: str) -> torch.Tensor:
        if name not in self.BUFFERS[self.name]:
            raise KeyError(f"buffer '{name}' of module '{self.name}': "
                           f"{list(self.BUFFERS[self.name])}")
        blk = self.block
        c = blk.options.coord()
        if name[0] == "x":
            d = int(name[1])
            f = c.faces(d)
            t = f if name.endswith("f") else 0.5 * (f[:-1] + f[1:])
            return torch.as_tensor(t, dtype=torch.float64, device=blk.device)
        b = blk.batch
        if name == "hydro_u":
            return b.current(0)
        if name == "u0":
            return b.store[0][b.rotation()[1]]
        if name == "scalar_s":
            s = b.current_scalars(0)
            if s is None:
                raise KeyError("buffer 'scalar_s': the block carries no scalars")
            return s
        if b.bases[0] is None:
            raise KeyError("buffer 'hydro_ref': the block stores totals")
        return b.bases[0]


class MeshBlock:
    """One block of the hydro stage on one GPU."""

    def __init__(self, options: MeshBlockOptions, tj: int = 0):
        self.options = options
        self._scheme = scheme_of(options)
        self._block = block_of(options, tj)
        self.intg = _Intg(options.intg())
        self.pintg = self.intg
        self.cycle = 0
        self.device = torch.device("cuda", torch.cuda.current_device()) \
            if torch.cuda.is_available() else torch.device("cpu")
        self.dtype = torch.float64 if options.hydro().precision == "float64" \
            else torch.float32
        self._batch: Optional[Batch] = None
        self._graphs: Dict[tuple, torch.cuda.CUDAGraph] = {}
        self._report = {"captures": 0, "replays": 0, "eager": 0, "graphs": 0,
                        "host": 0}
        self._seen = set()
        self._step_dims = set()  # the requested FluxRegister step fields

    # -- module-like API -----------------------------------------------------
    def to(self, device, dtype: Optional[torch.dtype] = None) -> "MeshBlock":
        device = torch.device(device)
        if device.type != "cuda":
            raise RuntimeError("snapy_gb300 runs on CUDA only; no CPU path")
        if device.index is None:
            device = torch.device("cuda", torch.cuda.current_device())
        self.device = device
        if dtype is not None:
            if dtype not in (torch.float32, torch.float64):
                raise ValueError(f"dtype {dtype}")
            self.dtype = dtype
        self._batch = None
        self._graphs.clear()
        self._seen.clear()
        return self

    @property
    def batch(self) -> Batch:
        if self._batch is None:
            self._batch = Batch(self._scheme, [self._block], self.device, self.dtype)
            if self.options.solve_corrections() != 2:
                self._batch.set_solve(self.options.solve_corrections())
            if self.options.sweep_mode():
                self._batch.set_sweep(self.options.sweep_mode())
            for d in sorted(self._step_dims):
                self._batch.request_step_field(0, d)
        return self._batch

    def flux_register(self) -> "FluxRegister":
        """The block's FluxRegister (HydroImpl::flux_register,
        src/hydro/hydro.hpp:135): its FP64 step fields."""
        return FluxRegister(self)

    def nc(self):
        c = self.options.coord()
        return (c.nc3, c.nc2, c.nc1)

    # -- reference API ---------------------------------------------------------
    def initialize(self, vars: dict):
        """Boundary functions on hydro_w (in place), hydro_u = W->U(hydro_w);
        with passive scalars, scalar_s = rho scalar_r (MeshBlockImpl::
        finalize_initialization, src/mesh/meshblock.cpp:380-383) from the
        required scalar_r (nscalar, nc3, nc2, nc1), ghosts by the boundary
        functions."""
        if "hydro_w" not in vars:
            raise RuntimeError("initialize: hydro_w is required for hydro model.")
        w = vars["hydro_w"]
        shape = (5,) + self.nc()
        if tuple(w.shape) != shape:
            raise RuntimeError(f"initialize: hydro_w has incorrect shape. "
                               f"Expected {list(shape)} but got {list(w.shape)}")
        if w.device != self.device:
            raise RuntimeError(f"initialize: hydro_w must be on {self.device}")
        if w.dtype != torch.float64:
            raise RuntimeError("initialize: hydro_w must be float64")
        if not w.is_contiguous():
            vars["hydro_w"] = w = w.contiguous()
        with torch.cuda.device(self.device):
            self.batch.init_from_prim([w])
            # integration/autotune: the tile width and finish form measured
            # on this block (not when the caller fixed the tile width)
            if self.options.autotune and not self._block.get("tj"):
                self.batch.autotune()
                self._graphs.clear()
                self._seen.clear()
            u = self.batch.current(0)
            ns = len(self.options.scalar_names)
            if ns:
                r = vars.get("scalar_r")
                if r is None:
                    raise RuntimeError("initialize: scalar_r is required")
                if tuple(r.shape) != (ns,) + self.nc():
                    raise RuntimeError("initialize: scalar_r has incorrect shape")
                # the conserved (dry) density of the initial state, FP64
                s = w[0].unsqueeze(0) * r.to(device=self.device, dtype=torch.float64)
                self.batch.init_scalars(0, s.to(self.dtype))
                sc = self.batch.current_scalars(0)
                vars["scalar_s"] = torch.empty(0, dtype=self.dtype,
                                               device=self.device).set_(sc)
        vars["hydro_u"] = torch.empty(0, dtype=self.dtype, device=self.device).set_(u)
        self.intg.current_redo = 0
        return vars, 0.0

    # -- module(name).buffer(name) (python/csrc/pyoptions.hpp:99-116) -------
    def buffer(self, name: str) -> torch.Tensor:
        """A named buffer of the block (the reference's named_buffers()):
        "hydro_u" (the current state), "u0" (the stage-0 state, MeshBlock's
        backup), "scalar_s", the coordinate's "x1f", "x1v", "x2f", "x2v",
        "x3f", "x3v" (FP64, ghosts included) and, for a block stored as
        anomalies, "hydro_ref" (its FP64 hydrostatic base)."""
        return _BlockModule(self, "").buffer(name)

    def module(self, name: str) -> "_BlockModule":
        """A named submodule (the reference's named_modules()): "hydro" or
        "coord" (or "" for the block), whose buffer(name) gives the
        buffers above that belong to it."""
        if name not in _BlockModule.BUFFERS:
            raise KeyError(f"module '{name}': the block has "
                           f"{sorted(k for k in _BlockModule.BUFFERS if k)}")
        return _BlockModule(self, name)

    # -- restart (src/output/restart.cpp, src/mesh/meshblock_restart.cpp) ---
    def write_restart(self, vars: dict, out_dir: str, basename: str = "snapy",
                      number: int = 0, time: float = 0.0, final: bool = False,
                      rank: int = 0, combine: bool = True, budget=None,
                      budget_fires: bool = False) -> str:
        """Write this block's restart part (RestartOutput::write_output_file,
        src/output/restart.cpp:40-140) and, with `combine`, the restart
        file of the parts present (combine_blocks); returns its path (the
        part's without `combine`).  Every tensor of vars is written on the
        CPU; hydro_u holds the conserved totals, and a block stored as
        anomalies about an FP64 hydrostatic base adds the stored bits, the
        base and the metadata [version, bits] with the grid faces.  With a
        budget consumer, its open interval goes along as the budget carry
        (BudgetOutput::save_carry, src/output/budget_series.cpp:224-227;
        budget_fires: the budget records at this time in the same pass); a
        carry read back from an earlier restart is not written again."""
        from . import restart as R
        from .budget import CARRY_PREFIX, write_budget_carry
        os.makedirs(out_dir, exist_ok=True)
        with torch.cuda.device(self.device):
            self._adopt(vars)
            out = {}
            skip_r = "scalar_s" in vars and "hydro_u" in vars
            for name, var in vars.items():
                if skip_r and name == "scalar_r":
                    continue
                if name.startswith(CARRY_PREFIX):
                    continue
                if isinstance(var, torch.Tensor) and var.numel():
                    out[name] = var.detach().cpu()
            u = self.batch.current(0)
            base = self.batch.bases[0]
            if base is not None:
                out["hydro_u"] = self.batch.totals(0, u).cpu()
                out["hydro_u_stored"] = u.detach().cpu().clone()
                out["hydro_ref"] = base.detach().cpu().clone()
                out[R.HYDRO_RESTART_METADATA] = torch.tensor(
                    [R.HYDRO_RESTART_VERSION, 32 if self.dtype == torch.float32 else 64],
                    dtype=torch.int64)
                c = self.options.coord()
                for d, key in enumerate(R.HYDRO_REFERENCE_GRID):
                    out[key] = torch.as_tensor(c.faces(d + 1), dtype=torch.float64)
            else:
                out["hydro_u"] = u.detach().cpu().clone()
            sc = self.batch.current_scalars(0)
            if sc is not None:
                out["scalar_s"] = sc.detach().cpu().clone()
        out["last_time"] = torch.tensor([float(time)], dtype=torch.float64)
        out["last_cycle"] = torch.tensor([int(self.cycle)], dtype=torch.int64)
        # the restart output's own schedule: its next file number and time
        out["file_number"] = torch.tensor([number + (0 if final else 1)],
                                          dtype=torch.int64)
        out["next_time"] = torch.tensor([float(time)], dtype=torch.float64)
        if budget is not None:
            write_budget_carry(budget.carry(self, vars, budget_fires), out)
        part = os.path.join(out_dir, R.part_name(basename, rank, number, final))
        R.save_part(out, part)
        return R.combine(out_dir, basename, number, final) if combine else part

    def initialize_from_restart(self, vars: dict, fname: str,
                                rank: int = 0, budget=None) -> float:
        """Resume from a restart file (MeshBlockImpl::_init_from_restart,
        src/mesh/meshblock_restart.cpp:33-236): the block's part, the
        required variables and the metadata checks; the cycle, the state
        (an anomaly block takes its stored bits and its FP64 base back, so
        the run continues bit for bit) and the tracers; vars gets every
        other variable of the file on the device.  With a budget consumer,
        its interval resumes from the file's budget carry when the carry's
        rows are the block's (BudgetOutput::load_carry); else it starts
        afresh at the next observe.  Returns the time."""
        from . import restart as R
        from .budget import ROWS, read_budget_carry
        data = R.load_restart(fname, rank)
        R.require(data)
        c = self.options.coord()
        R.check_restart_metadata(data, [c.faces(d) for d in (1, 2, 3)])
        shape = (5,) + self.nc()
        if tuple(data["hydro_u"].shape) != shape:
            raise R.RestartError(f"restart: hydro_u has shape "
                                 f"{tuple(data['hydro_u'].shape)}, the block {shape}")
        self.cycle = int(data["last_cycle"].item())
        t = float(data["last_time"].item())
        with torch.cuda.device(self.device):
            b = self.batch
            b.set_current(0)
            base = b.bases[0]
            if base is not None:
                if "hydro_ref" not in data or "hydro_u_stored" not in data:
                    raise R.RestartError("restart: an anomaly block needs "
                                         "hydro_ref and hydro_u_stored")
                stored = data["hydro_u_stored"]
                if stored.dtype != self.dtype or tuple(base.shape) != tuple(
                        data["hydro_ref"].shape):
                    raise R.RestartError("restart: the stored state's dtype or "
                                         "its base does not fit the block")
                base.copy_(data["hydro_ref"].to(self.device))
                b.current(0).copy_(stored.to(self.device))
            else:
                b.current(0).copy_(data["hydro_u"].to(self.device, self.dtype))
            sc = b.current_scalars(0)
            if sc is not None:
                if "scalar_s" not in data:
                    raise R.RestartError("restart: the block carries passive "
                                         "scalars; the file has no scalar_s")
                sc.copy_(data["scalar_s"].to(self.device, self.dtype))
                vars["scalar_s"] = torch.empty(0, dtype=self.dtype,
                                               device=self.device).set_(sc)
            skip = {"hydro_u", "hydro_u_stored", "hydro_ref", "scalar_s",
                    R.HYDRO_RESTART_METADATA, *R.HYDRO_REFERENCE_GRID}
            for name, tensor in data.items():
                if name not in skip:
                    vars[name] = tensor.to(self.device)
            vars["hydro_u"] = torch.empty(0, dtype=self.dtype,
                                          device=self.device).set_(b.current(0))
            self._graphs.clear()
            self._seen.clear()
            self.intg.current_redo = 0
            self._refresh_w(vars)
            if budget is not None:
                budget.resume(self, read_budget_carry(data, ROWS))
        return t

    def _publish(self, vars: dict) -> None:
        """vars views the block's current storage (hydro_u, scalar_s)."""
        b = self.batch
        vars["hydro_u"].set_(b.current(0))
        if "scalar_s" in vars and b.sstore[0] is not None:
            vars["scalar_s"].set_(b.current_scalars(0))

    def _adopt(self, vars: dict) -> None:
        u = vars.get("hydro_u")
        cur = self.batch.current(0)
        if u is None:
            raise RuntimeError("forward: vars has no hydro_u; call initialize")
        if u.data_ptr() != cur.data_ptr():
            cur.copy_(u)  # a rebound hydro_u is copied into block storage
            u.set_(cur)
            self._report["host"] += 1
        s = vars.get("scalar_s")
        sc = self.batch.current_scalars(0)
        if s is not None and sc is not None and s.data_ptr() != sc.data_ptr():
            sc.copy_(s)  # and a rebound scalar_s
            s.set_(sc)

    def forward(self, vars: dict, dt: float, stage: int) -> None:
        """One RK stage (MeshBlockImpl::forward, meshblock_advance.cpp:88).

        With execution auto / cuda-graph the stage's launches are captured
        once per (stage, buffer rotation) after an eager warm-up call and
        replayed; the dt is read from device memory, so one graph serves every
        dt (the reference's StepDt)."""
        nst = len(self.intg.stages)
        if not 0 <= stage < nst:
            raise RuntimeError(f"Invalid stage: {stage}")
        with torch.cuda.device(self.device):
            self._adopt(vars)
            b = self.batch
            b.dt.fill_(float(dt))
            rot = b.rotation()
            key = (stage,) + rot
            use_graph = self.options.execution != "eager"
            g = self._graphs.get(key) if use_graph else None
            if g is None and use_graph and key in self._seen:
                g = self._capture(stage, rot)
            if g is not None:
                g.replay()
                b.advance(stage)
                self._report["replays"] += 1
            else:
                b.stage(stage)
                self._seen.add(key)
                self._report["eager"] += 1
            self._publish(vars)

    def step(self, vars: dict, dt: float) -> None:
        """All stages of one step (the driver loop's ``for stage ...
        forward``), as ONE captured graph per buffer rotation when execution
        allows graphs.  Equal bit for bit to calling ``forward`` per stage."""
        nst = len(self.intg.stages)
        with torch.cuda.device(self.device):
            self._adopt(vars)
            b = self.batch
            b.dt.fill_(float(dt))
            rot = b.rotation()
            key = ("step",) + rot
            use_graph = self.options.execution != "eager"
            g = self._graphs.get(key) if use_graph else None
            if g is None and use_graph and key in self._seen:
                g = self._capture(None, rot)
            if g is not None:
                g.replay()
                for s in range(nst):
                    b.advance(s)
                self._report["replays"] += 1
            else:
                for s in range(nst):
                    b.stage(s)
                self._seen.add(key)
                self._report["eager"] += 1
            self._publish(vars)

    def _capture(self, stage, rot) -> torch.cuda.CUDAGraph:
        b = self.batch
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(device=self.device)
        s.wait_stream(torch.cuda.current_stream())
        try:
            with torch.cuda.stream(s):
                g.capture_begin()
                try:
                    if stage is None:
                        for st in range(len(self.intg.stages)):
                            b.stage(st)
                    else:
                        b.stage(stage)
                finally:
                    g.capture_end()
        finally:
            b.set_rotation(rot)  # the capture ran nothing: rewind the rotation
        torch.cuda.current_stream().wait_stream(s)
        self._graphs[("step" if stage is None else stage,) + tuple(rot)] = g
        self._report["captures"] += 1
        self._report["graphs"] = len(self._graphs)
        return g

    def max_time_step(self, vars: dict) -> float:
        with torch.cuda.device(self.device):
            self.batch.redo.fill_(self.intg.current_redo)
            dt = self.batch.max_dt()
            return float(dt[0].item())

    def check_redo(self, vars: dict) -> int:
        with torch.cuda.device(self.device):
            flags = int(self.batch.check()[0].item())
            if flags:
                self.batch.restore()
                self._publish(vars)
                self.intg.current_redo += 1
                self._refresh_w(vars)
                if self.intg.current_redo > self.intg.options.max_redo:
                    return -1
                return 1
            self.intg.current_redo = 0
            self._refresh_w(vars)
            return 0

    def _refresh_w(self, vars: dict) -> None:
        # "Retain the checked primitives for output and the next timestep"
        # (meshblock_redo.cpp:99-104): hydro_w <- W(hydro_u)
        w = vars.get("hydro_w")
        shape = (5,) + self.nc()
        if w is None or tuple(w.shape) != shape or w.device != self.device:
            vars["hydro_w"] = w = torch.empty(shape, dtype=torch.float64,
                                              device=self.device)
        if w.dtype == self.dtype:
            self.batch.prim([w])
        else:
            tmp = torch.empty(shape, dtype=self.dtype, device=self.device)
            self.batch.prim([tmp])
            w.copy_(tmp)

    def prim(self) -> torch.Tensor:
        """W of the current state (storage dtype)."""
        shape = (5,) + self.nc()
        out = torch.empty(shape, dtype=self.dtype, device=self.device)
        with torch.cuda.device(self.device):
            self.batch.prim([out])
        return out

    def total_u(self, vars) -> torch.Tensor:
        """The conserved totals: a copy of hydro_u, which in FP32 under
        gravity holds anomalies about the FP64 hydrostatic base, so there
        the base is added (the result is FP64)."""
        u = vars["hydro_u"] if isinstance(vars, dict) else vars
        if self.batch.bases[0] is not None:
            return self.batch.totals(0, u)
        return u.clone()

    def part(self, offset=(0, 0, 0), exterior: bool = True, extend_x1: int = 0,
             extend_x2: int = 0, extend_x3: int = 0):
        """Index of the interior (exterior=False) or of a neighbour slab, as
        MeshBlockImpl::part (src/mesh/meshblock.cpp:190-288) for offset 0."""
        c = self.options.coord()
        ng = c.nghost
        out = []
        for n, o, ext in ((c.nc3, offset[0], extend_x3), (c.nc2, offset[1], extend_x2),
                          (c.nc1, offset[2], extend_x1)):
            if n == 1:
                out.append(slice(0, 1, 1))
            elif o != 0:
                raise NotImplementedError("part: neighbour offsets are not built")
            else:
                out.append(slice(ng - ext, n - ng + ext, 1))
        return (slice(None),) + tuple(out)

    def execution_report(self) -> dict:
        return dict(self._report)

    def execution_capability(self, vars: dict) -> dict:
        seg = {"index": 0, "kind": "stage", "capturable": True,
               "reads_host_dt": False, "host": False,
               "ops": ["advance", "combine", "boundaries"], "reasons": []}
        fp64 = self.dtype == torch.float64
        return {"eager_fp64": fp64, "eager_fp32": not fp64, "graph_fp64": fp64,
                "graph_fp32": not fp64, "eager_reasons": [], "segments": [seg]}
