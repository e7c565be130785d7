"""Generate the golden face vectors from the reference's own kernels.

Run where the reference source tree is present (REFERENCE_ROOT, default: the
directory "reference" beside the repository): it builds
oracle/_ref/libsnapref.so from the reference's unmodified header-only
kernels (recon_point.h, riemann_kernels.h, ideal_gas_impl.h,
hydro_ref_x1_impl.h) and evaluates them on seeded random inputs. The output,
tests/golden/reference_faces.npz, travels with the repo so the oracle can be
pinned where the reference is absent.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_faces.npz")


SHALLOW = os.path.join(os.path.dirname(os.path.abspath(__file__)), "shallow_roe.npz")


def main_shallow(n=1000, seed=20261205):
    """The reference's shallow_roe_impl (src/riemann/riemann_kernels.h:447-495)
    with dir yz on seeded shallow-water states: geopotential in [50, 12000],
    velocities N(0, 30), for the x2 (dim 2) and x3 (dim 1) faces."""
    O.build()
    R = O.ref()
    if R is None:
        raise SystemExit("the reference shim was not built (no reference tree)")
    rng = np.random.default_rng(seed)
    wl = np.zeros((n, 4))
    wr = np.zeros((n, 4))
    for w in (wl, wr):
        w[:, 0] = rng.uniform(50.0, 12000.0, n)
        w[:, 1:] = rng.normal(0.0, 30.0, (n, 3))
    # equal states and tiny jumps too
    wr[: n // 10] = wl[: n // 10]
    wr[n // 10: n // 5] = wl[n // 10: n // 5] * (1 + 1e-9 * rng.normal(size=(n // 10, 4)))
    dims = np.array([2, 1])
    flux = np.zeros((2, n, 4))
    for di, dim in enumerate(dims):
        for i in range(n):
            a, b = np.ascontiguousarray(wl[i]), np.ascontiguousarray(wr[i])
            f = np.zeros(4)
            R.ref_shallow_roe(O.ptr(f), O.ptr(a), O.ptr(b), int(dim), 1)
            flux[di, i] = f
    np.savez_compressed(SHALLOW, wl=wl, wr=wr, dims=dims, flux=flux)
    print("wrote", SHALLOW)


def main(n=1000, seed=20261203):
    O.build()
    R = O.ref()
    if R is None:
        raise SystemExit("the reference shim was not built (no reference tree)")
    rng = np.random.default_rng(seed)
    # stencils: smooth, discontinuous, tiny and huge magnitudes, signs
    st = rng.normal(size=(n, 5)) * 10.0 ** rng.uniform(-4, 4, size=(n, 1))
    st[: n // 4] = np.abs(st[: n // 4])
    st[n // 4: n // 2, 2:] *= 1e3  # a jump inside the stencil
    weno = np.zeros((n, 2, 2))  # side (cm, cp) x scale (off, on)
    cp5 = np.zeros((n, 2))
    for k in range(n):
        s = np.ascontiguousarray(st[k])
        for side in (0, 1):
            cp5[k, side] = R.ref_cp5_point(O.ptr(s), side)
            for sc in (0, 1):
                weno[k, side, sc] = R.ref_weno5_point(O.ptr(s), side, sc)
    # Riemann states: Sod-like jumps, strong shocks, vacuum-ish expansions
    g = 1.4
    wl = np.zeros((n, 5))
    wr = np.zeros((n, 5))
    wl[:, 0] = 10 ** rng.uniform(-3, 1, n)
    wr[:, 0] = 10 ** rng.uniform(-3, 1, n)
    wl[:, 4] = 10 ** rng.uniform(-3, 3, n)
    wr[:, 4] = 10 ** rng.uniform(-3, 3, n)
    wl[:, 1:4] = rng.normal(size=(n, 3)) * 10 ** rng.uniform(-2, 1.5, (n, 1))
    wr[:, 1:4] = rng.normal(size=(n, 3)) * 10 ** rng.uniform(-2, 1.5, (n, 1))
    hllc = np.zeros((n, 3, 6))
    lmars = np.zeros((n, 3, 6))
    for k in range(n):
        a, b = wl[k].copy(), wr[k].copy()
        el, er = a[4] / (g - 1), b[4] / (g - 1)
        cl, cr = np.sqrt(g * a[4] / a[0]), np.sqrt(g * b[4] / b[0])
        hl, hr = a[4] / (g - 1) / a[0], b[4] / (g - 1) / b[0]
        for d, dim in enumerate((3, 2, 1)):
            f = np.zeros(5)
            p = np.zeros(1)
            R.ref_hllc(O.ptr(f), O.ptr(a.copy()), O.ptr(b.copy()), el, er, g, g,
                       cl, cr, dim, O.ptr(p))
            hllc[k, d, :5], hllc[k, d, 5] = f, p[0]
            R.ref_lmars(O.ptr(f), O.ptr(a.copy()), O.ptr(b.copy()), hl, hr, g, g,
                        dim, O.ptr(p))
            lmars[k, d, :5], lmars[k, d, 5] = f, p[0]
    # cons -> prim
    u = np.zeros((n, 5))
    u[:, 0] = wl[:, 0]
    u[:, 1:4] = wl[:, 1:4] * wl[:, :1]
    u[:, 4] = wl[:, 4] / (g - 1) + 0.5 * (u[:, 1:4] ** 2).sum(1) / u[:, 0] * 1.5
    prim = np.zeros((n, 5))
    for k in range(n):
        out = np.zeros(5)
        R.ref_cons2prim(O.ptr(out), O.ptr(u[k].copy()), g)
        prim[k] = out
    # hydrostatic face-pressure scan of random stratified columns
    nc1, iu = 70, 66
    cols = 8
    rho = np.exp(-np.linspace(0, 3, nc1))[None, :] * rng.uniform(0.5, 2, (cols, 1))
    scan = np.zeros((cols, 2, nc1))
    dx1f = np.full(nc1, 50.0)
    for c in range(cols):
        w = np.zeros((5, nc1))
        w[0] = rho[c]
        w[4] = 1e5 * rho[c]
        lo, hi = np.zeros(nc1), np.zeros(nc1)
        R.ref_pressure_scan(O.ptr(np.ascontiguousarray(w.ravel())), O.ptr(dx1f),
                            O.ptr(lo), O.ptr(hi), nc1, iu, -9.8)
        scan[c, 0], scan[c, 1] = lo, hi
    # the whole well-balanced x1 reference of stratified columns (uniform
    # grid, reflecting walls, wall clamp on): psf_lo, psf_hi, pref, dsf, dref
    ncol, nr = 6, 70
    zc = (np.arange(nr) - 2.5) * 50.0
    refcols = np.zeros((ncol, 5, nr))
    refw = np.zeros((ncol, 5, nr))
    for c in range(ncol):
        temp = 300.0 - 9.8 * zc / 1004.5 + rng.normal(size=nr) * c
        p = 1e5 * (temp / 300.0) ** 3.5
        w = np.zeros((5, nr))
        w[0], w[4] = p / (287.0 * temp), p
        w[1] = rng.normal(size=nr)
        w = np.ascontiguousarray(w)
        outs = [np.zeros(nr) for _ in range(5)]
        R.ref_hydro_ref_column(O.ptr(w.ravel()), O.ptr(np.full(nr, 50.0)),
                               *[O.ptr(o) for o in outs], nr, nr - 4, 9.8, 1, 1, 1)
        refw[c] = w
        refcols[c] = np.stack(outs)
    np.savez_compressed(OUT, stencils=st, weno=weno, cp5=cp5, wl=wl, wr=wr,
                        hllc=hllc, lmars=lmars, gammad=g, cons=u, prim=prim,
                        scan_rho=rho, scan=scan, scan_iu=iu, refw=refw,
                        refcols=refcols)
    print("wrote", OUT)


if __name__ == "__main__":
    if "--shallow" in sys.argv:
        main_shallow()
    else:
        main()
