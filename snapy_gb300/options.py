"""Deck options: ``MeshBlockOptions.from_yaml`` and the module option tables.

Mirrors the reference's option readers for the keys of the hydro-stage path
(src/mesh/meshblock_options.cpp:18-139, src/coord/coordinate.cpp:63-185,
src/eos/equation_of_state.cpp:60-142, src/recon/reconstruct.cpp:237-265,
src/riemann/riemann.cpp:55-76, src/options/hydro.yaml, pyharp's integrator
keys).  Unknown keys inside a section raise, as the reference's check_keys
does.  Keys the reference accepts but this stage does not implement are
accepted by the reader and refused by ``MeshBlock`` with a clear message.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field
from typing import Any, Dict, List, Optional

from . import yaml_lite

__all__ = [
    "CoordinateOptions", "EquationOfStateOptions", "ReconstructOptions",
    "RiemannSolverOptions", "GravityOptions", "DiffusionOptions",
    "ImplicitOptions", "HydroOptions", "IntegratorOptions",
    "MeshBlockOptions", "DeckError",
]


class DeckError(ValueError):
    """An invalid deck (the reference raises c10::Error -> RuntimeError)."""


def check_keys(node: Any, path: str, allowed) -> None:
    """src/input/check_keys.hpp: every key of `node` must be in `allowed`."""
    if node is None:
        return
    if not isinstance(node, dict):
        raise DeckError(f"{path} must be a map")
    bad = [k for k in node if k not in allowed]
    if bad:
        raise DeckError(f"{path}: unknown key(s) {bad}; allowed: {sorted(allowed)}")


def _get(node, key, default):
    if node is None or key not in node or node[key] is None:
        return default
    return node[key]


@dataclass
class CoordinateOptions:
    type: str = "cartesian"
    x1min: float = 0.0
    x1max: float = 1.0
    x2min: float = 0.0
    x2max: float = 1.0
    x3min: float = 0.0
    x3max: float = 1.0
    nx1: int = 1
    nx2: int = 1
    nx3: int = 1
    nghost: int = 1
    interp_order: int = 2

    def nc(self, n: int) -> int:
        return n + 2 * self.nghost if n > 1 else 1

    @property
    def nc1(self) -> int:
        return self.nc(self.nx1)

    @property
    def nc2(self) -> int:
        return self.nc(self.nx2)

    @property
    def nc3(self) -> int:
        return self.nc(self.nx3)

    @property
    def dx1(self) -> float:
        return (self.x1max - self.x1min) / self.nx1

    @property
    def dx2(self) -> float:
        return (self.x2max - self.x2min) / self.nx2

    @property
    def dx3(self) -> float:
        return (self.x3max - self.x3min) / self.nx3

    def faces(self, axis: int):
        """Global face coordinates of one axis, ghosts included, computed as
        the reference's block_faces_ (coordinate.cpp:410-425): a linspace over
        [min - ng dx, max + ng dx]."""
        import torch
        lo, hi, n = {1: (self.x1min, self.x1max, self.nx1),
                     2: (self.x2min, self.x2max, self.nx2),
                     3: (self.x3min, self.x3max, self.nx3)}[axis]
        if n <= 1:
            return torch.linspace(lo, hi, n + 1, dtype=torch.float64).numpy()
        dx = (hi - lo) / n
        ng = self.nghost
        return torch.linspace(lo - ng * dx, hi + ng * dx, n + 2 * ng + 1,
                              dtype=torch.float64).numpy()

    def centers(self, axis: int):
        f = self.faces(axis)
        return 0.5 * (f[:-1] + f[1:])

    @staticmethod
    def from_dict(config: dict) -> "CoordinateOptions":
        op = CoordinateOptions()
        g = config.get("geometry")
        if g is None:
            return op
        check_keys(g, "geometry", {"type", "bounds", "cells", "x1f", "x1rat"})
        if "x1f" in g or "x1rat" in g:
            op.type = g.get("type", op.type)
            raise DeckError("geometry: a stretched x1 (x1f / x1rat) is not "
                            "supported by this stage (uniform grids only)")
        op.type = _get(g, "type", op.type)
        b = g.get("bounds")
        check_keys(b, "geometry/bounds",
                   {"x1min", "x1max", "x2min", "x2max", "x3min", "x3max"})
        for k in ("x1min", "x1max", "x2min", "x2max", "x3min", "x3max"):
            if b and k in b:
                setattr(op, k, float(b[k]))
        c = g.get("cells")
        if c is None:
            op.nx1 = op.nx2 = op.nx3 = 1
            return op
        check_keys(c, "geometry/cells", {"nx1", "nx2", "nx3", "nghost",
                                         "interp_order", "interp-order"})
        op.nx1 = int(_get(c, "nx1", 1))
        op.nx2 = int(_get(c, "nx2", 1))
        op.nx3 = int(_get(c, "nx3", 1))
        op.nghost = int(_get(c, "nghost", 1))
        op.interp_order = int(_get(c, "interp_order", _get(c, "interp-order", 2)))
        for ax, n in ((1, op.nx1), (2, op.nx2), (3, op.nx3)):
            if n > 1 and n < op.nghost:
                raise DeckError(f"Number of x{ax} grids must be greater than "
                                "the ghost zone size")
        return op


@dataclass
class EquationOfStateOptions:
    type: str = "moist-mixture"
    gammad: float = 1.4
    weight: float = 29.e-3
    density_floor: float = 1.e-6
    pressure_floor: float = 1.e-3
    temperature_floor: float = 20.
    limiter: bool = False

    @staticmethod
    def from_dict(node) -> "EquationOfStateOptions":
        op = EquationOfStateOptions()
        if node is None:
            return op
        check_keys(node, "dynamics/equation-of-state",
                   {"type", "gammad", "weight", "density-floor",
                    "pressure-floor", "temperature-floor", "limiter",
                    "eos-file", "verbose", "max-iter", "ftol", "uv-solver"})
        op.type = _get(node, "type", op.type)
        op.gammad = float(_get(node, "gammad", op.gammad))
        op.weight = float(_get(node, "weight", op.weight))
        op.density_floor = float(_get(node, "density-floor", op.density_floor))
        op.pressure_floor = float(_get(node, "pressure-floor", op.pressure_floor))
        op.temperature_floor = float(_get(node, "temperature-floor",
                                          op.temperature_floor))
        op.limiter = bool(_get(node, "limiter", op.limiter))
        return op


@dataclass
class ReconstructOptions:
    type: str = "dc"
    scale: bool = False
    shock: bool = True

    @staticmethod
    def from_dict(node, path) -> "ReconstructOptions":
        op = ReconstructOptions()
        if node is None:
            return op
        check_keys(node, path, {"type", "scale", "shock"})
        op.type = _get(node, "type", op.type)
        op.scale = bool(_get(node, "scale", op.scale))
        op.shock = bool(_get(node, "shock", op.shock))
        return op


@dataclass
class RiemannSolverOptions:
    type: str = "hllc"
    dir: str = "xy"

    @staticmethod
    def from_dict(node) -> "RiemannSolverOptions":
        op = RiemannSolverOptions()
        if node is None:
            return op
        check_keys(node, "dynamics/riemann-solver", {"type", "dir"})
        op.type = _get(node, "type", op.type)
        op.dir = _get(node, "dir", op.dir)
        return op


@dataclass
class GravityOptions:
    grav1: float = 0.0
    grav2: float = 0.0
    grav3: float = 0.0
    non_hydrostatic: float = 1.0


@dataclass
class DiffusionOptions:
    nu_iso: float = 0.0
    nu_aniso: float = 0.0
    kappa: float = 0.0
    raw: dict = field(default_factory=dict)


@dataclass
class ImplicitOptions:
    scheme: int = 0
    precision: str = "auto"
    fallback_fp64: bool = True


_HYDRO_KEYS = {
    "equation-of-state", "reconstruct", "riemann-solver", "verbose",
    "disable-flux-x1", "disable-flux-x2", "disable-flux-x3", "wb-wall-clamp",
    "conversion-order", "anomaly", "flux-covariance", "x1-mass-covariance",
    "perturbation-flux", "precision", "conserve-axial-momentum",
}


@dataclass
class HydroOptions:
    eos: EquationOfStateOptions = field(default_factory=EquationOfStateOptions)
    recon1: ReconstructOptions = field(default_factory=ReconstructOptions)
    recon23: ReconstructOptions = field(default_factory=ReconstructOptions)
    riemann: RiemannSolverOptions = field(default_factory=RiemannSolverOptions)
    precision: str = "float64"
    flux_covariance: bool = True
    disable_flux: tuple = (False, False, False)
    anomaly: bool = False
    perturbation_flux: bool = False
    conversion_order: int = 2
    grav: Optional[GravityOptions] = None
    diffusion: Optional[DiffusionOptions] = None
    icorr: Optional[ImplicitOptions] = None
    extra: dict = field(default_factory=dict)

    @staticmethod
    def from_dict(config: dict) -> "HydroOptions":
        op = HydroOptions()
        dyn = config.get("dynamics")
        if dyn is not None:
            check_keys(dyn, "dynamics", _HYDRO_KEYS)
            op.eos = EquationOfStateOptions.from_dict(dyn.get("equation-of-state"))
            rec = dyn.get("reconstruct")
            check_keys(rec, "dynamics/reconstruct", {"vertical", "horizontal"})
            op.recon1 = ReconstructOptions.from_dict(
                rec.get("vertical") if rec else None, "dynamics/reconstruct/vertical")
            op.recon23 = ReconstructOptions.from_dict(
                rec.get("horizontal") if rec else None,
                "dynamics/reconstruct/horizontal")
            op.riemann = RiemannSolverOptions.from_dict(dyn.get("riemann-solver"))
            op.precision = str(_get(dyn, "precision", op.precision))
            if op.precision not in ("float64", "float32"):
                raise DeckError("dynamics/precision must be float64 or float32, "
                                f"got '{op.precision}'")
            op.flux_covariance = bool(_get(dyn, "flux-covariance", True))
            op.disable_flux = tuple(bool(_get(dyn, f"disable-flux-x{d}", False))
                                    for d in (1, 2, 3))
            env = os.environ.get("SNAP_ANOMALY")
            op.anomaly = bool(_get(dyn, "anomaly", False)) if env is None else env == "1"
            op.perturbation_flux = bool(_get(dyn, "perturbation-flux", False))
            op.conversion_order = int(_get(dyn, "conversion-order", 2))
            op.extra = {k: dyn[k] for k in ("x1-mass-covariance",
                                            "conserve-axial-momentum",
                                            "wb-wall-clamp") if k in dyn}
        forcing = config.get("forcing")
        if forcing is not None:
            cg = forcing.get("const-gravity")
            if cg is not None:
                check_keys(cg, "forcing/const-gravity",
                           {"grav1", "grav2", "grav3", "non-hydrostatic"})
                op.grav = GravityOptions(
                    grav1=float(_get(cg, "grav1", 0.)),
                    grav2=float(_get(cg, "grav2", 0.)),
                    grav3=float(_get(cg, "grav3", 0.)),
                    non_hydrostatic=float(_get(cg, "non-hydrostatic", 1.)))
            df = forcing.get("diffusion")
            if df is not None:
                op.diffusion = DiffusionOptions(
                    nu_iso=float(_get(df, "nu_iso", _get(df, "nu-iso", 0.))),
                    nu_aniso=float(_get(df, "nu_aniso", _get(df, "nu-aniso", 0.))),
                    kappa=float(_get(df, "kappa", 0.)), raw=dict(df))
        intg = config.get("integration")
        if intg is not None:
            scheme = int(_get(intg, "implicit-scheme", 0))
            prec = str(_get(intg, "implicit-precision", "auto"))
            if prec not in ("auto", "float32", "float64"):
                raise DeckError("integration/implicit-precision must be auto, "
                                f"float32 or float64, got '{prec}'")
            if scheme != 0:
                op.icorr = ImplicitOptions(
                    scheme=scheme, precision=prec,
                    fallback_fp64=bool(_get(intg, "implicit-fallback-fp64", True)))
            elif prec != "auto":
                op.icorr = None
        return op


_RK_WEIGHTS = {
    # (w0, w1, w2) per stage: u <- w0 u0 + w1 u + w2 du (Shu-Osher forms;
    # w2 pinned by the reference's tests/test_forcing.cpp:1316-1322)
    "rk1": [(1., 0., 1.)],
    "rk2": [(1., 0., 1.), (.5, .5, .5)],
    "rk3": [(1., 0., 1.), (3. / 4., 1. / 4., 1. / 4.), (1. / 3., 2. / 3., 2. / 3.)],
}


@dataclass
class IntegratorWeight:
    wght0: float
    wght1: float
    wght2: float


@dataclass
class IntegratorOptions:
    type: str = "rk3"
    cfl: float = 0.9
    tlim: float = 0.0
    nlim: int = -1
    ncycle_out: int = 1
    max_redo: int = 5

    @property
    def stages(self) -> List[IntegratorWeight]:
        if self.type not in _RK_WEIGHTS:
            raise DeckError(f"integration/type '{self.type}' is not supported")
        return [IntegratorWeight(*w) for w in _RK_WEIGHTS[self.type]]

    @staticmethod
    def from_dict(config) -> "IntegratorOptions":
        op = IntegratorOptions()
        node = config.get("integration")
        if node is None:
            return op
        check_keys(node, "integration",
                   {"type", "cfl", "tlim", "nlim", "ncycle_out", "max-redo",
                    "max_redo", "implicit-scheme", "implicit-precision",
                    "implicit-fallback-fp64", "execution", "execution-strict",
                    "restart", "autotune", "implicit-solve",
                    "implicit-corrections", "implicit-sweep"})
        op.type = str(_get(node, "type", op.type))
        op.cfl = float(_get(node, "cfl", op.cfl))
        op.tlim = float(_get(node, "tlim", op.tlim))
        op.nlim = int(_get(node, "nlim", op.nlim))
        op.ncycle_out = int(_get(node, "ncycle_out", op.ncycle_out))
        op.max_redo = int(_get(node, "max-redo", _get(node, "max_redo", op.max_redo)))
        return op


_TOP_KEYS = {"reference-state", "species", "geometry", "distribute", "dynamics",
             "boundary-condition", "integration", "outputs", "forcing",
             "problem", "scalar", "verbose", "sedimentation", "chemistry"}
_BC_NAMES = {"reflecting", "periodic", "extrapolation", "outflow", "custom",
             "solid", "fixed_temperature"}


def _scalar_names(node, op) -> List[str]:
    """The passive scalars of the deck's scalar section
    (ScalarOptionsImpl::from_yaml, src/scalar/scalar_options.cpp): the
    transport is built without the upper bound and with the upwind solver
    and the hydro's WENO5 (scale-invariant, as the reference always
    reconstructs a scalar)."""
    if not node:
        return []
    check_keys(node, "scalar", {"verbose", "nvar", "upper-bound", "names",
                                "reconstruct", "riemann-solver"})
    names = [str(x) for x in (node.get("names") or [])]
    nvar = int(node.get("nvar", len(names)))
    if not names:
        names = [f"scalar{n}" for n in range(nvar)]
    if float(node.get("upper-bound", -1.0)) > 0.0:
        raise DeckError("scalar/upper-bound: the upper-bound limiter is not built")
    rs = node.get("riemann-solver")
    if rs and str((rs or {}).get("type", "upwind")) != "upwind":
        raise DeckError("scalar/riemann-solver: only upwind is built")
    rc = node.get("reconstruct")
    if rc and str((rc or {}).get("type", "weno5")) != "weno5":
        raise DeckError("scalar/reconstruct: only weno5 is built")
    if names:
        h, c = op.hydro(), op.coord()
        if h.eos.type == "shallow-water":
            raise DeckError("scalar: passive scalars need a dry-air density")
    return names


SWEEPS = {"serial": 0, "partitioned": 1, "auto": 2}


def shared_sweep(modes) -> int:
    """The one sg_set_sweep mode of blocks batched in a handle: the serial
    sweep if any block asks for it (its results are bit for bit the
    reference's order), the partitioned form if every block asks for it,
    else the autotuner's choice."""
    modes = list(modes)
    if 0 in modes:
        return 0
    return 1 if all(m == 1 for m in modes) else 2


def shared_solve(ks) -> int:
    """The one solve form of blocks batched in a handle, from their decks'
    sg_set_solve arguments: the direct FP64 solve if any block asks for it,
    else the refined solve with the fewest corrections any block asks for,
    else the FP32 solve."""
    ks = list(ks)
    if 0 in ks:
        return 0
    pos = [k for k in ks if k > 0]
    return min(pos) if pos else -1


class MeshBlockOptions:
    """The deck of one block (reference MeshBlockOptionsImpl)."""

    def solve_corrections(self) -> int:
        """sg_set_solve's argument for this deck: 0 for the direct FP64
        solve, -1 for the FP32 solve, else the refined solve's corrections."""
        if self.implicit_solve == "direct":
            return 0
        if self.implicit_solve == "fp32":
            return -1
        return self.implicit_corrections

    def sweep_mode(self) -> int:
        """sg_set_sweep's argument for this deck."""
        return SWEEPS[self.implicit_sweep]

    def __init__(self):
        self._coord = CoordinateOptions()
        self._hydro = HydroOptions()
        self._intg = IntegratorOptions()
        self.bcnames: List[str] = []
        self.execution = "auto"
        self.execution_strict = False
        # integration/autotune (no counterpart in the reference): time the
        # stage's tile widths and finish forms on the block at initialize
        self.autotune = True
        # integration/implicit-solve (no counterpart in the reference): the
        # solve of implicit-precision float32 blocks, "refined" (FP32 sweeps
        # corrected with FP64 residuals to the FP64 solution), "direct" (the
        # FP64 solve of every column) or "fp32" (the reference's own FP32
        # compute: the FP32 sweep alone, the FP64 retry of failed columns);
        # scheme 9's only: scheme 1's FP32-assembled 3x3 blocks are solved
        # directly in FP64
        self.implicit_solve = "refined"
        self.implicit_corrections = 2  # FP64-residual corrections (1 to 3)
        # integration/implicit-sweep (no counterpart in the reference): the
        # order of elimination of the scheme-9 solve of FP64-assembled
        # blocks, "serial" (the reference's column sweep, bit for bit),
        # "partitioned" (each column in four chunks swept at once and a
        # separator system, for batches with few columns; the same solution
        # to rounding) or "auto" (the autotuner times both)
        self.implicit_sweep = "serial"
        # scalar/nvar, scalar/names: passive scalars (ScalarOptionsImpl,
        # src/scalar/scalar.hpp)
        self.scalar_names: List[str] = []
        self.verbose = False
        self.basename = ""
        self.problem: Dict[str, Any] = {}
        self.config: Dict[str, Any] = {}

    # reference-style accessors: opts.coord(), opts.coord(new)
    def coord(self, value: Optional[CoordinateOptions] = None):
        if value is not None:
            self._coord = value
        return self._coord

    def hydro(self, value: Optional[HydroOptions] = None):
        if value is not None:
            self._hydro = value
        return self._hydro

    def intg(self, value: Optional[IntegratorOptions] = None):
        if value is not None:
            self._intg = value
        return self._intg

    def device_str(self) -> str:
        return "cuda"

    def __repr__(self) -> str:
        c = self._coord
        return (f"MeshBlockOptions(coord={c.type} {c.nx3}x{c.nx2}x{c.nx1}, "
                f"riemann={self._hydro.riemann.type}, "
                f"precision={self._hydro.precision}, execution={self.execution})")

    @staticmethod
    def from_yaml(filename: str, verbose: bool = False) -> "MeshBlockOptions":
        config = yaml_lite.load(filename) or {}
        return MeshBlockOptions.from_config(config, filename, verbose)

    @staticmethod
    def from_config(config: dict, filename: str = "", verbose: bool = False):
        check_keys(config, "<deck>", _TOP_KEYS)
        op = MeshBlockOptions()
        op.config = config
        base = os.path.basename(filename)
        op.basename = base.rsplit(".", 1)[0] if "." in base else base
        op._hydro = HydroOptions.from_dict(config)
        op._intg = IntegratorOptions.from_dict(config)
        op.verbose = bool(config.get("verbose", verbose))
        intg = config.get("integration") or {}
        op.execution = str(intg.get("execution", "auto"))
        op.execution_strict = bool(intg.get("execution-strict", False))
        op.autotune = bool(intg.get("autotune", True))
        op.implicit_solve = str(intg.get("implicit-solve", "refined"))
        if op.implicit_solve not in ("refined", "direct", "fp32"):
            raise DeckError("integration/implicit-solve must be refined, "
                            f"direct or fp32, got '{op.implicit_solve}'")
        op.implicit_sweep = str(intg.get("implicit-sweep", "serial"))
        if op.implicit_sweep not in SWEEPS:
            raise DeckError("integration/implicit-sweep must be serial, "
                            f"partitioned or auto, got '{op.implicit_sweep}'")
        op.implicit_corrections = int(intg.get("implicit-corrections", 2))
        if not 1 <= op.implicit_corrections <= 3:
            raise DeckError("integration/implicit-corrections must be 1 to 3, "
                            f"got {op.implicit_corrections}")
        if op.execution not in ("auto", "eager", "cuda-graph"):
            raise DeckError("integration/execution must be auto, eager or "
                            f"cuda-graph, got '{op.execution}'")
        if op.execution == "eager" and op.execution_strict:
            raise DeckError("integration/execution-strict needs execution: "
                            "cuda-graph (eager is never refused)")
        op._coord = CoordinateOptions.from_dict(config)
        op.scalar_names = _scalar_names(config.get("scalar"), op)
        op.problem = dict(config.get("problem") or {})
        bcs = config.get("boundary-condition")
        if bcs is not None:
            check_keys(bcs, "boundary-condition", {"external", "internal"})
            ext = bcs.get("external")
            if ext is not None:
                check_keys(ext, "boundary-condition/external",
                           {"x1-inner", "x1-outer", "x2-inner", "x2-outer",
                            "x3-inner", "x3-outer"})
                ns = [op._coord.nc1, op._coord.nc2, op._coord.nc3]
                for d in range(3):
                    if ns[d] <= 1:
                        above = (d == 0 and (ns[1] > 1 or ns[2] > 1)) or (
                            d == 1 and ns[2] > 1)
                        if above:
                            op.bcnames += ["", ""]
                        continue
                    for side in ("inner", "outer"):
                        name = str(ext.get(f"x{d + 1}-{side}", "reflecting"))
                        if name not in _BC_NAMES:
                            raise DeckError(f"Boundary function '{name}_{side}' "
                                            "is not defined.")
                        op.bcnames.append(f"{name}_{side}")
        return op
