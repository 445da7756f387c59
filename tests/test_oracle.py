"""The FP64 oracle pinned against the reference's own host code (golden
fixtures from oracle/_ref) and 50-digit Fourier-integral values."""
import numpy as np
import pytest

import oracle


def test_scalar_functions_match_reference(golden):
    g = golden["ref_scalar"]
    for i in range(len(g["r2"])):
        r2, a, d = g["r2"][i], g["a"][i], g["d"][i]
        for j, fn in enumerate((oracle.diffH, oracle.regH)):
            h = np.array(fn(r2, a, d))
            np.testing.assert_allclose(h, g["H"][i, j], rtol=1e-13, atol=1e-300)
            hl = np.array(fn(0.0, a, d))
            np.testing.assert_allclose(hl, g["lim"][i, j], rtol=1e-13)
    ex = [oracle.lib().pbo_experf(x, z, 2.0) for x, z in zip(g["ex_x"], g["ex_z"])]
    np.testing.assert_allclose(ex, g["experf"], rtol=1e-14, atol=0)


def test_pair_tensors_match_reference(golden):
    g = golden["ref_scalar"]
    for i in range(len(g["r2"])):
        A = oracle.vR(g["xh"][i], g["a"][i], g["d"][i], g["e"][i]).reshape(-1, order="F")
        np.testing.assert_allclose(A, g["vR"][i], rtol=1e-12, atol=1e-14 * np.abs(g["vR"][i]).max())
        F = oracle.vF(g["xh"][i], g["a"][i], g["d"][i], g["k"][i]).reshape(-1, order="F")
        np.testing.assert_allclose(F, g["vF"][i], rtol=1e-12, atol=1e-14 * np.abs(g["vF"][i]).max())


@pytest.mark.parametrize("case", ["iso_self", "aniso", "singular", "converged", "converged_aniso"])
def test_shell_matrix_matches_reference(golden, case):
    g = golden["ref_shells"]
    a, d, e, M, N = g[case + "_par"]
    Mx, Nx = oracle.shell_counts(g[case + "_L"], int(M), int(N))
    np.testing.assert_array_equal(Mx, g[case + "_Mx"])
    np.testing.assert_array_equal(Nx, g[case + "_Nx"])
    A = oracle.shell_matrix(g[case + "_x"], g[case + "_x0"], a, d, e, Mx, Nx, g[case + "_L"])
    ref = g[case + "_A"]
    assert np.abs(A - ref).max() <= 1e-12 * np.abs(ref).max()


def test_shell_counts_by_hand():
    # P.h:457-487: real shells shrink along the longer axes, Fourier shells grow.
    Mx, Nx = oracle.shell_counts([1.0, 1.0, 1.0], 3, 5)
    assert list(Mx) == [3, 3, 3] and list(Nx) == [5, 5, 5]
    Mx, Nx = oracle.shell_counts([1.0, 2.0, 4.0], 4, 3)
    assert list(Mx) == [4, 2, 1] and list(Nx) == [12, 6, 3]
    Mx, Nx = oracle.shell_counts([0.8, 1.0, 1.3], 2, 10)
    assert list(Mx) == [2, 2, 2] and list(Nx) == [17, 13, 10]


def test_accurate_kernel_vs_mpmath(golden):
    rows = golden["mp_kernel"]["rows"]
    for a, d, e, r, h1, h2 in rows:
        H = oracle.pair_H(r, a, d, e)
        scale1 = abs(oracle.pair_H(0.0, a, d, e)[0]) if e > 0 else 1.0 / (8 * np.pi * max(r, 1e-3 * d))
        assert abs(H[0] - h1) <= 1e-12 * max(abs(h1), scale1), (a, d, e, r, H, h1)
        # H2 multiplies x x^T: compare on the scale of H2 * r^2 against H1
        assert abs(H[1] - h2) * max(r * r, 1e-30) <= 1e-12 * max(abs(h1), scale1) + 1e-12 * abs(h2) * r * r, (a, d, e, r)


def test_converged_ewald_matches_reference_shells(golden):
    g = golden["ref_shells"]
    for case in ("converged", "converged_aniso"):
        a, d, e, M, N = g[case + "_par"]
        A = g[case + "_A"]
        f = g[case + "_f"]
        u_ref = (A @ f.reshape(-1)).reshape(-1, 3)
        u = oracle.ewald_velocity(g[case + "_x"], g[case + "_x0"], f, g[case + "_L"], a, e, d=d)
        mx, rms = oracle.rel_errors(u, u_ref)
        assert mx < 1e-11, (case, mx)


@pytest.mark.parametrize("alpha,eps", [(7.0, 0.01), (7.0, 0.0), (1.0, 0.005), (40.0, 0.002)])
def test_splitting_independence(alpha, eps):
    # the total real + k-space sum does not depend on the splitting blob
    # (the invariant studied by the reference driver, cuda/periodicBrinkman.cu:139-194)
    rng = np.random.default_rng(5)
    n = 60
    L = np.array([1.0, 1.2, 0.9])
    x = rng.random((n, 3)) * L
    f = rng.standard_normal((n, 3))
    us = [oracle.ewald_velocity(x, x, f, L, alpha, eps, d=d) for d in (0.05, 0.08, 0.12, 0.2)]
    for u in us[1:]:
        assert oracle.rel_errors(u, us[0])[0] < 2e-12


def test_periodicity_and_translation():
    rng = np.random.default_rng(6)
    n = 40
    L = np.array([1.0, 1.0, 1.0])
    x = rng.random((n, 3))
    f = rng.standard_normal((n, 3))
    u0 = oracle.ewald_velocity(x, x, f, L, 10.0, 0.02, d=0.12)
    shift = rng.integers(-2, 3, (n, 3)) * L
    u1 = oracle.ewald_velocity(x, x + shift, f, L, 10.0, 0.02, d=0.12)
    assert oracle.rel_errors(u1, u0)[0] < 1e-12
    t = np.array([0.31, -0.17, 0.42])
    u2 = oracle.ewald_velocity(x + t, x + t, f, L, 10.0, 0.02, d=0.12)
    assert oracle.rel_errors(u2, u0)[0] < 1e-12


def test_zero_mode_and_empty():
    x = np.array([[0.1, 0.2, 0.3]])
    f = np.array([[1.0, -2.0, 0.5]])
    L = np.array([1.0, 2.0, 1.5])
    u0 = oracle.ewald_velocity(x, x, f, L, 4.0, 0.01, d=0.1)
    u1 = oracle.ewald_velocity(x, x, f, L, 4.0, 0.01, d=0.1, zero_mode=True)
    np.testing.assert_allclose(u1 - u0, f / (16.0 * 3.0), rtol=0, atol=1e-13 * np.abs(u0).max())
    assert oracle.ewald_velocity(np.zeros((0, 3)), x, f, L, 4.0, 0.01, d=0.1).shape == (0, 3)
