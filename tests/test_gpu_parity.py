"""GPU parity: every GPU path through the C ABI against the FP64 oracle and
the reference's own outputs (golden fixtures)."""
import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import periodicbrinkman_gb300 as pb  # noqa: E402
from periodicbrinkman_gb300.api import Plan, make_params  # noqa: E402


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


@pytest.fixture(scope="module", autouse=True)
def _device():
    assert torch.cuda.is_available()
    assert pb.device_count() > 0


# ---------------------------------------------------------------- dense matrix
@pytest.mark.parametrize("case", ["iso_self", "aniso", "singular", "converged", "converged_aniso"])
def test_dense_matrix_matches_reference(golden, case):
    g = golden["ref_shells"]
    a, d, e, M, N = g[case + "_par"]
    x, x0 = g[case + "_x"], g[case + "_x0"]
    m, n = x.shape[0], x0.shape[0]
    dA = torch.zeros((3 * n, 3 * m), dtype=torch.float64, device="cuda").t()  # column-major (3m, 3n)
    pb.periodicBrinkman(dA, cuda(x), cuda(x0), a, d, e, int(M), int(N), g[case + "_L"])
    A = dA.cpu().numpy()
    ref = g[case + "_A"]
    assert np.abs(A - ref).max() <= 1e-12 * np.abs(ref).max(), np.abs(A - ref).max() / np.abs(ref).max()


def test_dense_matrix_accumulates_and_skips(golden):
    g = golden["ref_shells"]
    a, d, e, M, N = g["aniso_par"]
    x, x0 = g["aniso_x"], g["aniso_x0"]
    m, n = x.shape[0], x0.shape[0]
    base = torch.full((3 * n, 3 * m), 0.5, dtype=torch.float64, device="cuda").t()
    pb.periodicBrinkman(base, cuda(x), cuda(x0), a, d, e, int(M), int(N), g["aniso_L"])
    assert np.abs(base.cpu().numpy() - 0.5 - g["aniso_A"]).max() <= 1e-12 * np.abs(g["aniso_A"]).max()
    # M < 0 and N = 0 leave dA untouched
    z = torch.zeros((3 * n, 3 * m), dtype=torch.float64, device="cuda").t()
    pb.periodicBrinkman(z, cuda(x), cuda(x0), a, d, e, -1, 0, g["aniso_L"])
    assert float(z.abs().max()) == 0.0


# ---------------------------------------------------------------- evaluator
def _case(n, L, seed, m=0):
    rng = np.random.default_rng(seed)
    L = np.asarray(L, dtype=np.float64)
    x = rng.random((n, 3)) * L
    f = rng.standard_normal((n, 3))
    y = rng.random((m, 3)) * L if m else None
    return x, f, y


@pytest.mark.parametrize("prec,tol,bound", [("fp64", 1e-10, 1e-9), ("mixed", 1e-6, 1e-6)])
@pytest.mark.parametrize("alpha,eps", [(10.0, 0.01), (1.0, 0.005), (40.0, 0.02), (5.0, 0.0)])
def test_solve_matches_oracle(prec, tol, bound, alpha, eps):
    x, f, _ = _case(700, 1.0, 11)
    u = pb.solve(cuda(x), cuda(f), 1.0, alpha, eps, tol=tol, precision=prec).cpu().numpy()
    u_ref = oracle.ewald_velocity(x, x, f, 1.0, alpha, eps)
    mx, rms = oracle.rel_errors(u, u_ref)
    assert mx < bound, (prec, alpha, eps, mx, rms)


@pytest.mark.parametrize("prec,bound", [("fp64", 1e-9), ("mixed", 1e-6)])
def test_solve_separate_targets_anisotropic(prec, bound):
    L = np.array([1.0, 0.7, 1.4])
    x, f, y = _case(600, L, 12, m=350)
    u = pb.solve(cuda(x), cuda(f), L, 8.0, 0.01, y=cuda(y), tol=1e-10 if prec == "fp64" else 1e-6,
                 precision=prec).cpu().numpy()
    u_ref = oracle.ewald_velocity(y, x, f, L, 8.0, 0.01)
    assert oracle.rel_errors(u, u_ref)[0] < bound


def test_host_and_device_buffers_agree():
    # spreading accumulates with atomics, so repeated solves agree to rounding, not bitwise
    x, f, _ = _case(300, 1.0, 13)
    u_h = pb.solve(x, f, 1.0, 10.0, 0.01, precision="fp64", tol=1e-10)
    u_d = pb.solve(cuda(x), cuda(f), 1.0, 10.0, 0.01, precision="fp64", tol=1e-10).cpu().numpy()
    assert np.abs(u_h - u_d).max() <= 1e-13 * np.abs(u_h).max()


def test_graph_replay_is_stable():
    x, f, _ = _case(800, 1.0, 14)
    p = make_params(800, 1.0, 10.0, 0.01, tol=1e-6, precision="mixed")
    with Plan(p) as plan:
        xs, fs = cuda(x), cuda(f)
        outs = [plan.execute(xs, fs).clone() for _ in range(4)]  # eager, capture, replay, replay
        assert plan.kernel_count > 10
    for o in outs[1:]:
        assert float((o - outs[0]).abs().max()) <= 1e-6 * float(outs[0].abs().max())


def test_zero_mode_and_flags():
    x, f, _ = _case(200, (1.0, 2.0, 1.5), 15)
    L = np.array([1.0, 2.0, 1.5])
    base = pb.solve(cuda(x), cuda(f), L, 4.0, 0.01, precision="fp64", tol=1e-10).cpu().numpy()
    zm = pb.solve(cuda(x), cuda(f), L, 4.0, 0.01, precision="fp64", tol=1e-10, flags=7).cpu().numpy()
    np.testing.assert_allclose(zm - base, np.tile(f.sum(0) / (16.0 * 3.0), (200, 1)), rtol=0,
                               atol=1e-11 * np.abs(base).max())
    # real-only + k-only == both
    pr = make_params(200, L, 4.0, 0.01, tol=1e-10, precision="fp64")
    r_only = pb.solve(cuda(x), cuda(f), L, 4.0, 0.01, precision="fp64", tol=1e-10, flags=1, d=0.2).cpu().numpy()
    k_only = pb.solve(cuda(x), cuda(f), L, 4.0, 0.01, precision="fp64", tol=1e-10, flags=2, d=0.2).cpu().numpy()
    both = pb.solve(cuda(x), cuda(f), L, 4.0, 0.01, precision="fp64", tol=1e-10, d=0.2).cpu().numpy()
    np.testing.assert_allclose(r_only + k_only, both, rtol=0, atol=1e-12 * np.abs(both).max())
    assert pr.n_src == 200
    # the split parts agree with the oracle's split parts
    kr = oracle.ewald_velocity(x, x, f, L, 4.0, 0.01, d=0.2, real=False)
    assert oracle.rel_errors(k_only, kr)[0] < 1e-8


def test_fft_brinkman_kspace_matches_oracle():
    x, f, y = _case(400, 1.0, 16, m=120)
    U = np.zeros((120, 3))
    # the reference's parameters: grid 64^3, P = 16 support points, m = 7 standard deviations
    # (truncation ~exp(-(7*7/8)^2/2), aliasing ~exp(-pi^2 P^2/(2 m^2)))
    pb.fftBrinkman(U, y, f, x, [1, 1, 1], [64, 64, 64], [16, 16, 16], 7, 0, 0.01, 1e-6, 0.125, 10.0)
    kr = oracle.ewald_velocity(y, x, f, 1.0, 10.0, 0.01, d=0.125, real=False)
    assert oracle.rel_errors(U, kr)[0] < 1e-7


def test_batch_equals_individual_solves():
    rng = np.random.default_rng(17)
    params, xs, fs, us = [], [], [], []
    for k in range(5):
        n = int(rng.integers(100, 600))
        L = rng.uniform(0.5, 2.0)
        a = float(np.exp(rng.uniform(0, np.log(50))))
        x = rng.random((n, 3)) * L
        f = rng.standard_normal((n, 3))
        p = make_params(n, L, a, 0.01 * L, tol=1e-6, precision="mixed")
        params.append(p)
        xs.append(x)
        fs.append(f)
        us.append(pb.solve(cuda(x), cuda(f), L, a, 0.01 * L, tol=1e-6, precision="mixed").cpu().numpy())
    with Plan(params) as plan:
        U = plan.execute(cuda(np.concatenate(xs)), cuda(np.concatenate(fs))).cpu().numpy()
    off = 0
    for k in range(5):
        n = xs[k].shape[0]
        ref = us[k]
        assert np.abs(U[off:off + n] - ref).max() <= 1e-6 * np.abs(ref).max()
        off += n


def test_config1_parameters_error_reported():
    # N = 1000, alpha = 10, eps = 0.01, xi = 8 (d = 0.125), rc = 0.35, 64^3, P = 16
    x, f, _ = _case(1000, 1.0, 1000)
    u64 = pb.solve(cuda(x), cuda(f), 1.0, 10.0, 0.01, d=0.125, rc=0.35, M=64, P=16, precision="fp64").cpu().numpy()
    umx = pb.solve(cuda(x), cuda(f), 1.0, 10.0, 0.01, d=0.125, rc=0.35, M=64, P=16, precision="mixed").cpu().numpy()
    u_ref = oracle.ewald_velocity(x, x, f, 1.0, 10.0, 0.01)
    e64 = oracle.rel_errors(u64, u_ref)[0]
    emx = oracle.rel_errors(umx, u_ref)[0]
    # the fixed cutoff 0.35 = 2.8 d truncates the real-space sum at ~1e-4 of the near field
    assert e64 < 1e-3 and emx < 1e-3
    assert oracle.rel_errors(umx, u64)[0] < 1e-6


@pytest.mark.parametrize("M,L,d,rc,P", [(8, 1.0, 0.25, 0.45, 4), (16, 1.0, 0.15, 0.4, 6), (32, 1.0, 0.1, 0.3, 8),
                                        (128, 1.0, 0.03, 0.11, 10), (256, 1.0, 0.02, 0.075, 12),
                                        ((32, 64, 16), (1.0, 2.0, 0.5), 0.08, 0.25, 8)])
def test_mixed_matches_fp64_on_every_fft_length(M, L, d, rc, P):
    """The FP32 k-space path (register FFT passes for lines of 4..256 points,
    anisotropic grids included) agrees with the FP64 path on the same
    splitting, cutoff, grid and support."""
    Ls = L if isinstance(L, tuple) else (L, L, L)
    Ms = M if isinstance(M, tuple) else (M, M, M)
    rng = np.random.default_rng(sum(Ms))
    x = rng.random((400, 3)) * np.array(Ls)
    f = rng.standard_normal((400, 3))
    kw = dict(d=d, rc=rc, M=Ms, P=P, tol=1e-6)
    u64 = pb.solve(cuda(x), cuda(f), L, 10.0, 0.01, precision="fp64", **kw).cpu().numpy()
    umx = pb.solve(cuda(x), cuda(f), L, 10.0, 0.01, precision="mixed", **kw).cpu().numpy()
    assert np.abs(umx - u64).max() <= 2e-6 * np.abs(u64).max()


def test_empty_and_invalid():
    x, f, _ = _case(10, 1.0, 18)
    with pytest.raises(pb.PbError):
        pb.solve(cuda(x), cuda(f), 1.0, -1.0, 0.01)
    bad = x.copy()
    bad[3, 1] = np.nan
    with pytest.raises(pb.PbError):
        pb.solve(bad, f, 1.0, 10.0, 0.01)
    u = pb.solve(cuda(np.zeros((0, 3))), cuda(np.zeros((0, 3))), 1.0, 10.0, 0.01, y=cuda(x)).cpu().numpy()
    assert u.shape == (10, 3) and np.all(u == 0)


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_host_non_finite_inputs_found_on_device(prec):
    """Host-memory executions find non-finite positions, forces and targets
    through the device flags; the plan stays usable and matches a clean run."""
    from periodicbrinkman_gb300 import _lib

    x, f, y = _case(300, 1.0, 19, m=120)
    p = make_params(300, 1.0, 10.0, 0.01, n_tgt=120, tol=1e-6, precision=prec)
    with Plan(p) as plan:
        ref = plan.execute(x, f, y=y)
        for arr, idx, val in ((x, (5, 0), np.nan), (f, (7, 2), np.inf), (y, (3, 1), -np.inf)):
            bad = arr.copy()
            bad[idx] = val
            args = dict(x=x, f=f, y=y)
            args["x" if arr is x else "f" if arr is f else "y"] = bad
            with pytest.raises(pb.PbError) as ei:
                plan.execute(args["x"], args["f"], y=args["y"])
            assert ei.value.code == _lib.PB_ERR_INVALID
        again = plan.execute(x, f, y=y)
    # atomics make the summation order vary between runs: equal to rounding
    assert np.abs(again - ref).max() <= 1e-6 * np.abs(ref).max()


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_item_capacity_overflow_is_an_error(prec):
    """Real-space work items beyond the plan's item array are reported (an
    error, not silently dropped pairs), on host and device buffers; at full
    capacity the same plan runs clean again."""
    from periodicbrinkman_gb300 import _lib

    x, f, _ = _case(4000, 1.0, 23)
    p = make_params(4000, 1.0, 10.0, 0.01, tol=1e-6, precision=prec)
    with Plan(p) as plan:
        ref = plan.execute(x, f)
        full = 4 * 4000 + 4096
        plan.set_item_capacity(8)
        with pytest.raises(pb.PbError) as ei:
            plan.execute(x, f)
        assert ei.value.code == _lib.PB_ERR_UNSUPPORTED and "item capacity" in str(ei.value)
        plan.execute(cuda(x), cuda(f))
        with pytest.raises(pb.PbError) as ei:
            plan.status()
        assert ei.value.code == _lib.PB_ERR_UNSUPPORTED
        plan.set_item_capacity(full)
        again = plan.execute(x, f)
        plan.status()
    assert np.abs(again - ref).max() <= 1e-6 * np.abs(ref).max()
