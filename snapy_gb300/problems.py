"""Initial states of the decks this stage serves (the reference's example
drivers: examples/shock.cpp for Sod, examples/straka.cpp for the density
current), as FP64 primitive tensors ``hydro_w`` of shape (5, nc3, nc2, nc1).
"""
from __future__ import annotations

import math
from typing import Optional

import torch

from .options import MeshBlockOptions

RGAS = 8.31446261815324  # kintera constants::Rgas (J/mol/K)


def _centers(options: MeshBlockOptions, axis: int, device) -> torch.Tensor:
    c = options.coord()
    return torch.tensor(c.centers(axis), dtype=torch.float64, device=device)


def sod(options: MeshBlockOptions, device="cuda") -> torch.Tensor:
    """Sod shock tube along x1 (problem keys x0, rho_l, p_l, rho_r, p_r)."""
    c = options.coord()
    p = options.problem
    x0 = float(p.get("x0", 0.5))
    x1v = _centers(options, 1, device)
    w = torch.zeros((5, c.nc3, c.nc2, c.nc1), dtype=torch.float64, device=device)
    left = (x1v < x0).view(1, 1, -1)
    w[0] = torch.where(left, float(p.get("rho_l", 1.0)), float(p.get("rho_r", 0.125)))
    w[4] = torch.where(left, float(p.get("p_l", 1.0)), float(p.get("p_r", 0.1)))
    return w


def ensemble_members(n: int = 64, seed: int = 20261203,
                     deck: str = "straka.yaml", precision: Optional[str] = None,
                     nx2_choices=(128, 256, 384, 512),
                     nx1_choices=(32, 64, 96, 128), dx: float = 50.0,
                     device="cpu"):
    """Members of a Straka-type ensemble: member k draws, from a generator
    seeded with seed + k, its size (nx2, nx1) uniformly from the choices, a
    bubble amplitude dT ~ U[-20, -10] K, a centre xc ~ U[0, 0.25 Lx],
    zc ~ U[0.3, 0.6] Lz, and radii min(4 km, 0.15 Lx), min(2 km, 0.3 Lz).
    Returns [(options, hydro_w)]."""
    import os
    path = deck if os.path.isabs(deck) else os.path.join(
        os.path.dirname(os.path.abspath(__file__)), "decks", deck)
    out = []
    for k in range(n):
        g = torch.Generator().manual_seed(seed + k)
        pick = lambda seq: seq[int(torch.randint(len(seq), (1,), generator=g))]
        nx2, nx1 = pick(nx2_choices), pick(nx1_choices)
        u = torch.rand(3, generator=g, dtype=torch.float64)
        opts = MeshBlockOptions.from_yaml(path)
        c = opts.coord()
        c.nx1, c.nx2 = nx1, nx2
        c.x1max, c.x2max = nx1 * dx, nx2 * dx
        if precision:
            opts.hydro().precision = precision
        Lx, Lz = nx2 * dx, nx1 * dx
        w = straka(opts, device, dT=-20.0 + 10.0 * float(u[0]),
                   xc=0.25 * Lx * float(u[1]), zc=(0.3 + 0.3 * float(u[2])) * Lz,
                   xr=min(4.e3, 0.15 * Lx), zr=min(2.e3, 0.3 * Lz))
        out.append((opts, w))
    return out


def straka(options: MeshBlockOptions, device="cuda", dT=None, xc=None, zc=None,
           xr=None, zr=None) -> torch.Tensor:
    """Straka density current (examples/straka.cpp:133-186): an isentropic
    base state of potential temperature Ts over p0 and a cosine cold bubble
    of amplitude dT centred at (xc, zc) with radii (xr, zr); x1 is vertical."""
    c = options.coord()
    p = options.problem
    eos = options.hydro().eos
    grav = -options.hydro().grav.grav1 if options.hydro().grav else 9.8
    p0 = float(p.get("p0", 1.e5))
    Ts = float(p.get("Ts", 300.))
    xc = float(p.get("xc", 0.) if xc is None else xc)
    xr = float(p.get("xr", 4.e3) if xr is None else xr)
    zc = float(p.get("zc", 3.e3) if zc is None else zc)
    zr = float(p.get("zr", 2.e3) if zr is None else zr)
    dT = float(p.get("dT", -15.) if dT is None else dT)
    Rd = RGAS / eos.weight
    cv = Rd / (eos.gammad - 1.)  # IdealGasImpl::species_cv_ref
    cp = cv + Rd
    x1v = _centers(options, 1, device).view(1, 1, -1)
    x2v = _centers(options, 2, device).view(1, -1, 1)
    L = torch.sqrt(((x2v - xc) / xr).square() + ((x1v - zc) / zr).square())
    temp = (Ts - grav * x1v / cp).expand(c.nc3, c.nc2, c.nc1)
    w = torch.zeros((5, c.nc3, c.nc2, c.nc1), dtype=torch.float64, device=device)
    # the pressure is the unperturbed isentrope; the bubble changes rho only
    w[4] = p0 * torch.pow(temp / Ts, cp / Rd)
    temp = temp + torch.where(L <= 1, dT * (torch.cos(L * math.pi) + 1.) / 2.,
                              torch.zeros_like(L))
    w[0] = w[4] / (Rd * temp)
    return w


def convection3d(options: MeshBlockOptions, device="cuda", seed: int = 0) -> torch.Tensor:
    """3-D planar dry convection at rest: the isentropic base state of
    potential temperature Ts over p0 (as straka's) with potential-temperature
    noise dtheta U[-1, 1], drawn from a generator seeded with `seed`, in the
    cells whose centre lies in the lowest `layer` fraction of the x1 extent
    (problem keys p0, Ts, dtheta, layer); x1 is vertical."""
    c = options.coord()
    p = options.problem
    eos = options.hydro().eos
    grav = -options.hydro().grav.grav1 if options.hydro().grav else 9.8
    p0 = float(p.get("p0", 1.e5))
    Ts = float(p.get("Ts", 300.))
    dtheta = float(p.get("dtheta", 0.1))
    layer = float(p.get("layer", 0.1))
    Rd = RGAS / eos.weight
    cv = Rd / (eos.gammad - 1.)
    cp = cv + Rd
    x1v = _centers(options, 1, device).view(1, 1, -1)
    temp = (Ts - grav * x1v / cp).expand(c.nc3, c.nc2, c.nc1)
    w = torch.zeros((5, c.nc3, c.nc2, c.nc1), dtype=torch.float64, device=device)
    w[4] = p0 * torch.pow(temp / Ts, cp / Rd)
    g = torch.Generator().manual_seed(int(seed))
    noise = (2. * torch.rand((c.nc3, c.nc2, c.nc1), generator=g,
                             dtype=torch.float64) - 1.) * dtheta
    low = (x1v - c.x1min) < layer * (c.x1max - c.x1min)
    noise = torch.where(low.cpu(), noise, torch.zeros_like(noise)).to(device)
    w[0] = w[4] / (Rd * temp * (1. + noise / Ts))
    return w
