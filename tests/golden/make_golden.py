"""Generate the golden fixtures in tests/golden/ (run here, where the
reference tree and mpmath exist; the .npz outputs are committed).

  ref_scalar.npz   experf/singH/regH/diffH/vR/vF from the reference's own host
                   code (cuda/periodicBrinkman.h:19-208), compiled from its
                   sources by oracle/build_ref.sh into oracle/_ref/.
  ref_shells.npz   dense mobility matrices from the reference's realShells +
                   fourierShells (cuda/periodicBrinkman.h:564-823) called the
                   way its driver calls them (cuda/periodicBrinkman.cu:176-182).
  mp_kernel.npz    50-digit mpmath values of the regularized-Brinkmanlet
                   difference R_e - R_d and of S - R_d from the radial Fourier
                   integral of the modified-blob symbol, at radii where the
                   closed forms lose digits.

Usage:  python tests/golden/make_golden.py
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import oracle  # noqa: E402

dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)


def P(a):
    return a.ctypes.data_as(dp)


def make_ref_scalar(R):
    rng = np.random.default_rng(20150419)
    n = 400
    r2 = 10 ** rng.uniform(-6, 0.3, n)
    a = 10 ** rng.uniform(0, 1.7, n)
    d = 10 ** rng.uniform(-2.5, -0.3, n)
    H = np.zeros((n, 3, 2))
    for i in range(n):
        for j, fn in enumerate((R.ref_diffH, R.ref_regH)):
            out = np.zeros(2)
            fn(r2[i], a[i], d[i], P(out))
            H[i, j] = out
        out = np.zeros(2)
        R.ref_singH(r2[i], a[i], P(out))
        H[i, 2] = out
    # r -> 0 limits (r below the switch radius)
    lim = np.zeros((n, 2, 2))
    for i in range(n):
        for j, fn in enumerate((R.ref_diffH, R.ref_regH)):
            out = np.zeros(2)
            fn(0.0, a[i], d[i], P(out))
            lim[i, j] = out
    ex_x = rng.uniform(-5, 5, n)
    ex_z = rng.uniform(-30, 30, n)
    experf = np.array([R.ref_experf(ex_x[i], ex_z[i], 2.0) for i in range(n)])
    xh = rng.uniform(-1, 1, (n, 3)) * 10 ** rng.uniform(-3, 0, (n, 1))
    e = np.where(rng.random(n) < 0.2, 0.0, d * 10 ** rng.uniform(-1.5, 0, n))
    vR = np.zeros((n, 9))
    vF = np.zeros((n, 9))
    k = 2 * np.pi * rng.integers(-12, 13, (n, 3)) / rng.uniform(0.5, 2.0, (n, 3))
    k[np.all(k == 0, axis=1)] = [2 * np.pi, 0, 0]
    for i in range(n):
        out = np.zeros(9)
        R.ref_vR(P(out), P(np.ascontiguousarray(xh[i])), a[i], d[i], e[i])
        vR[i] = out
        out = np.zeros(9)
        R.ref_vF(P(out), P(np.ascontiguousarray(xh[i])), a[i], d[i], P(np.ascontiguousarray(k[i])))
        vF[i] = out
    np.savez_compressed(os.path.join(HERE, "ref_scalar.npz"), r2=r2, a=a, d=d, H=H, lim=lim, ex_x=ex_x, ex_z=ex_z,
                        experf=experf, xh=xh, e=e, vR=vR, k=k, vF=vF)


SHELL_CASES = [
    # name, m, n, same, L, alpha, d, eps, M, N
    ("iso_self", 8, 8, True, (1.0, 1.0, 1.0), 10.0, 0.125, 0.01, 2, 6),
    ("aniso", 7, 5, False, (1.0, 1.3, 0.8), 5.0, 0.2, 0.02, 1, 4),
    ("singular", 6, 6, False, (1.0, 1.0, 1.0), 3.0, 0.3, 0.0, 1, 3),
    ("converged", 12, 12, True, (1.0, 1.0, 1.0), 10.0, 0.125, 0.01, 2, 18),
    ("converged_aniso", 9, 9, True, (1.0, 0.7, 1.4), 20.0, 0.1, 0.005, 2, 32),
]


def make_ref_shells(R):
    rng = np.random.default_rng(1014)
    out = {}
    for name, m, n, same, L, a, d, e, M, N in SHELL_CASES:
        L = np.array(L)
        x0 = rng.random((n, 3)) * L
        x = x0.copy() if same else rng.random((m, 3)) * L
        f = rng.standard_normal((n, 3))
        Mx, Nx = oracle.shell_counts(L, M, N)
        A = np.zeros(9 * m * n)
        R.ref_shells(P(A), P(np.ascontiguousarray(x)), m, P(np.ascontiguousarray(x0)), n, Mx.ctypes.data_as(ip),
                     Nx.ctypes.data_as(ip), P(L), a, d, e)
        out[name + "_x"] = x
        out[name + "_x0"] = x0
        out[name + "_f"] = f
        out[name + "_L"] = L
        out[name + "_par"] = np.array([a, d, e, M, N])
        out[name + "_Mx"] = Mx
        out[name + "_Nx"] = Nx
        out[name + "_A"] = A.reshape(3 * m, 3 * n, order="F")
    np.savez_compressed(os.path.join(HERE, "ref_shells.npz"), **out)


def make_mp_kernel():
    import mpmath as mp

    mp.mp.dps = 50

    def phihat(k, a, d):
        x = a * a * d * d
        a1 = 1 - mp.e ** (-x / 4)
        return (1 + a1 * k * k / (a * a)) * mp.e ** (-k * k * d * d / 4)

    def s1(z):
        if z == 0:
            return mp.mpf(2) / 3
        j0 = mp.sin(z) / z
        j1 = mp.sin(z) / z ** 2 - mp.cos(z) / z
        return j0 - j1 / z

    def s2(z):
        if z == 0:
            return mp.mpf(1) / 15
        j2 = (3 / z ** 2 - 1) * mp.sin(z) / z - 3 * mp.cos(z) / z ** 2
        return j2 / z ** 2

    def R(r, a, d1, d2):
        """R_d1 - R_d2 (d2 = None: R_d1 alone)."""
        def ph(k):
            v = phihat(k, a, d1)
            if d2 is not None:
                v -= phihat(k, a, d2)
            return v
        dm = d1 if d2 is None else min(d1, d2)
        pts = [0] + [mp.mpf(j) / dm for j in (1, 2, 4, 8, 16)] + [mp.inf]
        h1 = mp.quad(lambda k: ph(k) * k * k / (k * k + a * a) * s1(k * r), pts)
        h2 = mp.quad(lambda k: ph(k) * k ** 4 / (k * k + a * a) * s2(k * r), pts)
        return h1 / (2 * mp.pi ** 2), h2 / (2 * mp.pi ** 2)

    def S(r, a):
        u = a * r
        A1 = (-1 + mp.e ** (-u) * (1 + u + u * u)) / u ** 2
        A2 = (3 - mp.e ** (-u) * (3 + 3 * u + u * u)) / u ** 2
        return A1 / (4 * mp.pi * r), A2 / (4 * mp.pi * r ** 3)

    rows = []
    cases = [(10.0, 0.125, 0.01), (1.0, 0.05, 0.005), (50.0, 0.02, 0.002), (20.0, 0.3, 0.03), (3.0, 0.1, 0.0)]
    for a, d, e in cases:
        a_, d_, e_ = mp.mpf(a), mp.mpf(d), mp.mpf(e)
        for rr in (0.0, 1e-4, 0.01, 0.05, 0.15, 0.3, 1.0, 2.5):
            r = rr * (e if e > 0 else d)
            if e == 0 and r == 0:
                h = R(mp.mpf(0), a_, d_, None)
                h = (-h[0], -h[1])
            elif e > 0:
                h = R(mp.mpf(r), a_, e_, d_)
            else:
                Rd = R(mp.mpf(r), a_, d_, None)
                Sv = S(mp.mpf(r), a_)
                h = (Sv[0] - Rd[0], Sv[1] - Rd[1])
            rows.append((a, d, e, r, float(h[0]), float(h[1])))
    np.savez_compressed(os.path.join(HERE, "mp_kernel.npz"), rows=np.array(rows))


def main():
    oracle.build_ref()
    R = oracle.ref_lib()
    if R is None:
        print("reference not available; ref fixtures not regenerated")
    else:
        make_ref_scalar(R)
        make_ref_shells(R)
    make_mp_kernel()
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
