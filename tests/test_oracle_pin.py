"""Pin the CPU oracle against the reference's own kernels.

The golden vectors in tests/golden/reference_faces.npz were produced by the
reference's unmodified header-only kernels (tests/golden/make_golden.py).  The
oracle's restatement must reproduce them bit for bit.  Where the reference
tree is present (oracle/_ref built), fresh random cases are compared too.
"""
import ctypes

import numpy as np
import pytest


def test_weno5_cp5_golden(oracle, golden):
    L = oracle.lib()
    st = golden["stencils"]
    for k in range(st.shape[0]):
        s = np.ascontiguousarray(st[k])
        for side in (0, 1):
            assert L.og_cp5_face(oracle.ptr(s), side) == golden["cp5"][k, side]
            for sc in (0, 1):
                got = L.og_weno5_face(oracle.ptr(s), side, sc)
                want = golden["weno"][k, side, sc]
                assert got == want or (np.isnan(got) and np.isnan(want)), (k, side, sc)


@pytest.mark.parametrize("solver", ["hllc", "lmars"])
def test_riemann_golden(oracle, golden, solver):
    L = oracle.lib()
    fn = L.og_hllc_face if solver == "hllc" else L.og_lmars_face
    g = float(golden["gammad"])
    wl, wr, ref = golden["wl"], golden["wr"], golden[solver]
    for k in range(wl.shape[0]):
        a, b = np.ascontiguousarray(wl[k]), np.ascontiguousarray(wr[k])
        for d, dim in enumerate((3, 2, 1)):
            f = np.zeros(5)
            p = np.zeros(1)
            fn(oracle.ptr(a), oracle.ptr(b), g, dim, oracle.ptr(f), oracle.ptr(p))
            np.testing.assert_array_equal(f, ref[k, d, :5])
            assert p[0] == ref[k, d, 5]


def test_cons2prim_golden(oracle, golden):
    L = oracle.lib()
    u, prim = golden["cons"], golden["prim"]
    for k in range(u.shape[0]):
        w = np.zeros(5)
        L.og_cons2prim_cell(oracle.ptr(np.ascontiguousarray(u[k])), oracle.ptr(w),
                            float(golden["gammad"]), 1)
        np.testing.assert_array_equal(w, prim[k])


def test_fresh_cases_against_reference_build(oracle):
    R = oracle.ref()
    if R is None:
        pytest.skip("reference tree not present: golden vectors only")
    L = oracle.lib()
    rng = np.random.default_rng(7)
    for _ in range(3000):
        s = rng.normal(size=5) * 10 ** rng.uniform(-3, 3)
        for side in (0, 1):
            for sc in (0, 1):
                assert L.og_weno5_face(oracle.ptr(s), side, sc) == \
                    R.ref_weno5_point(oracle.ptr(s), side, sc)
        wl = np.array([rng.uniform(.1, 2), *rng.normal(size=3), rng.uniform(.1, 2)])
        wr = np.array([rng.uniform(.1, 2), *rng.normal(size=3), rng.uniform(.1, 2)])
        g = 1.4
        for dim in (1, 2, 3):
            f1, f2, p1, p2 = np.zeros(5), np.zeros(5), np.zeros(1), np.zeros(1)
            L.og_hllc_face(oracle.ptr(wl), oracle.ptr(wr), g, dim, oracle.ptr(f1),
                           oracle.ptr(p1))
            R.ref_hllc(oracle.ptr(f2), oracle.ptr(wl.copy()), oracle.ptr(wr.copy()),
                       wl[4] / (g - 1), wr[4] / (g - 1), g, g,
                       np.sqrt(g * wl[4] / wl[0]), np.sqrt(g * wr[4] / wr[0]), dim,
                       oracle.ptr(p2))
            np.testing.assert_array_equal(f1, f2)


def test_reference_column_golden(oracle, golden):
    """The well-balanced x1 reference of a column (face pressures, cell
    pressure, face and cell densities) against the reference's own kernel.
    The anchor's exp is the oracle's portable one (libm's differs by at most
    an ulp), hence a 1e-15 relative bound instead of bit equality."""
    L = oracle.lib()
    refw, refcols = golden["refw"], golden["refcols"]
    nr = refw.shape[-1]
    b = oracle.Block(nc1=nr, dx1=50.0, grav1=-9.8,
                     bc=("reflecting", "reflecting", "none", "none", "none", "none"))
    for c in range(refw.shape[0]):
        w = np.ascontiguousarray(refw[c])
        outs = [np.zeros(nr) for _ in range(5)]
        dlr = np.zeros(2 * nr)
        L.og_ref_column(ctypes.byref(b.b), oracle.ptr(w.ravel()), nr,
                        *[oracle.ptr(o) for o in outs], oracle.ptr(dlr))
        for k in range(5):
            np.testing.assert_allclose(outs[k], refcols[c, k], rtol=1e-15, atol=0)


def test_portable_exp_within_an_ulp(oracle):
    L = oracle.lib()
    L.og_exp.restype = ctypes.c_double
    L.og_exp.argtypes = [ctypes.c_double]
    import math
    for x in np.concatenate([np.linspace(-0.05, 0.05, 4001), np.linspace(-600, 600, 4001)]):
        a, b = L.og_exp(float(x)), math.exp(float(x))
        assert abs(a - b) <= math.ulp(b), x
