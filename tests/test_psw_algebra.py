"""The algebra of the partitioned column solve (vic_psolve_kernel), restated
in numpy and checked against a dense solve of the same block-tridiagonal
system: four chunks separated by three single separator layers, each chunk
swept top-down with the left separator's coupling as extra right-hand
sides, the backward recurrence that writes every layer in terms of its two
separators, the separators' own 3-row system, then every layer.  Every
chunk remainder of n - 3 layers over four chunks is covered (n = 16 to 19),
and the lengths the benchmarks use.  The kernel's own results are checked
against the oracle on the GPU (tests/test_gpu_psolve.py); this pins the
equations it implements."""
import numpy as np
import pytest

P = 4  # chunks per column


def dense(A, B, C, r):
    n = len(A)
    M = np.zeros((5 * n, 5 * n))
    for i in range(n):
        M[5 * i:5 * i + 5, 5 * i:5 * i + 5] = A[i]
        if i > 0:
            M[5 * i:5 * i + 5, 5 * i - 5:5 * i] = B[i]
        if i < n - 1:
            M[5 * i:5 * i + 5, 5 * i + 5:5 * i + 10] = C[i]
    return np.linalg.solve(M, r.reshape(5 * n, -1)).reshape(n, 5, -1)


def chunks(n):
    """(first layer, layers) of each chunk, as the kernel lays them out."""
    m = n - (P - 1)
    lb, lr = divmod(m, P)
    return [(g * (lb + 1) + min(g, lr), lb + (1 if g < lr else 0)) for g in range(P)]


def partitioned(A, B, C, r):
    n = len(A)
    ch = chunks(n)
    Y, E, F, cpe, vpe, ye = {}, {}, {}, {}, {}, {}
    for g, (s0, L) in enumerate(ch):
        Cp, Vp, y = {}, {}, {}
        for t in range(L):
            i = s0 + t
            M, rhs, V = A[i].copy(), r[i].copy(), np.zeros((5, 5))
            if t == 0:
                if g > 0:
                    V = -B[i]  # the left separator's coupling
            else:
                M = M - B[i] @ Cp[i - 1]
                rhs = rhs - B[i] @ y[i - 1]
                V = -B[i] @ Vp[i - 1]
            Cp[i] = np.linalg.solve(M, C[i])
            y[i] = np.linalg.solve(M, rhs)
            Vp[i] = np.linalg.solve(M, V)
        e = s0 + L - 1
        cpe[g], vpe[g], ye[g] = Cp[e], Vp[e], y[e]
        Eg = {e: np.zeros((5, 5)) if g == P - 1 else -Cp[e]}
        Fg, Yg = {e: Vp[e]}, {e: y[e]}
        for i in range(e - 1, s0 - 1, -1):
            Eg[i] = -Cp[i] @ Eg[i + 1]
            Fg[i] = Vp[i] - Cp[i] @ Fg[i + 1]
            Yg[i] = y[i] - Cp[i] @ Yg[i + 1]
        Y[g], E[g], F[g] = Yg, Eg, Fg
    seps = [s0 + L for s0, L in ch[:-1]]
    Ah, Bh, Ch, rh = [], [], [], []
    for p, sg in enumerate(seps):
        s1 = ch[p + 1][0]
        Ah.append(A[sg] - B[sg] @ cpe[p] + C[sg] @ F[p + 1][s1])
        Bh.append(B[sg] @ vpe[p])
        Ch.append(C[sg] @ E[p + 1][s1])
        rh.append(r[sg] - B[sg] @ ye[p] - C[sg] @ Y[p + 1][s1])
    xs = dense(Ah, Bh, Ch, np.array(rh))
    x = np.zeros_like(r)
    for p, sg in enumerate(seps):
        x[sg] = xs[p]
    for g, (s0, L) in enumerate(ch):
        xr = xs[g] if g < P - 1 else np.zeros_like(r[0])
        xl = xs[g - 1] if g > 0 else np.zeros_like(r[0])
        for i in range(s0, s0 + L):
            x[i] = Y[g][i] + E[g][i] @ xr + F[g][i] @ xl
    return x


def test_layout_covers_every_layer_once():
    for n in range(16, 200):
        ch = chunks(n)
        seps = [s0 + L for s0, L in ch[:-1]]
        layers = sorted(sum((list(range(s0, s0 + L)) for s0, L in ch), []) + seps)
        assert layers == list(range(n)), n
        assert min(L for _, L in ch) >= 3


@pytest.mark.parametrize("n", [16, 17, 18, 19, 32, 64, 96, 128])
def test_partitioned_equals_dense(n):
    rng = np.random.default_rng(n)
    A = np.eye(5) * 4 + rng.normal(size=(n, 5, 5))
    B = rng.normal(size=(n, 5, 5)) * 0.5
    C = rng.normal(size=(n, 5, 5)) * 0.5
    B[0] = 0.0      # no layer below the first
    C[n - 1] = 0.0  # nor above the last
    r = rng.normal(size=(n, 5, 3))  # three right-hand sides, as d, z0, z1
    x0 = dense(A, B, C, r)
    x1 = partitioned(A, B, C, r)
    assert np.abs(x1 - x0).max() <= 1e-12 * np.abs(x0).max()
