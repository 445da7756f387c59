"""The C-ABI library loads, exports every symbol of include/pbrinkman.h, and
its host-side logic (parameter validation, autotuner, kernel tables) works
without a GPU."""
import ctypes as C

import numpy as np
import pytest

import oracle
import periodicbrinkman_gb300 as pb
from periodicbrinkman_gb300 import _lib
from periodicbrinkman_gb300.api import estimate_bytes, make_params, resolve


def test_library_exports_header_symbols():
    L = pb.lib()
    names = _lib.header_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n


def test_version_and_device_count():
    assert b"sm_103a" in pb.lib().pb_version()
    assert pb.device_count() >= 0


@pytest.mark.skipif(_lib.device_count() > 0, reason="checks the no-GPU error path")
def test_compute_entry_points_fail_loudly_without_gpu():
    p = make_params(10, 1.0, 10.0, 0.01)
    x = np.random.default_rng(0).random((10, 3))
    with pytest.raises(pb.PbError) as ei:
        pb.solve(x, x.copy(), 1.0, 10.0, 0.01)
    assert ei.value.code == _lib.PB_ERR_CUDA
    U = np.zeros((4, 3))
    with pytest.raises(pb.PbError):
        pb.fftBrinkman(U, x[:4].copy(), x.copy(), x.copy(), [1, 1, 1], [16, 16, 16], [8, 8, 8], 4, 0, 0.01, 1e-6,
                       0.1, 10.0)
    assert p.n_src == 10


@pytest.mark.parametrize("bad", [
    dict(L=(1.0, 0.0, 1.0)), dict(alpha=0.0), dict(eps=-1e-3), dict(alpha=float("nan")), dict(L=(1, float("inf"), 1)),
    dict(tol=2.0), dict(M=(64, 60, 64)), dict(P=7), dict(P=40), dict(precision=5), dict(flags=64),
])
def test_invalid_parameters_rejected(bad):
    kw = dict(L=(1.0, 1.0, 1.0), alpha=10.0, eps=0.01)
    kw.update(bad)
    p = make_params(100, kw.pop("L"), kw.pop("alpha"), kw.pop("eps"), **kw)
    with pytest.raises(pb.PbError) as ei:
        estimate_bytes(p)
    assert ei.value.code in (_lib.PB_ERR_INVALID, _lib.PB_ERR_UNSUPPORTED)


def test_autotuner_resolves_consistent_parameters():
    for n, L, a, e, tol, prec in [(1000, 1.0, 10.0, 0.01, 1e-6, "mixed"), (100000, 1.0, 20.0, 0.005, 1e-6, "mixed"),
                                  (100000, 1.0, 20.0, 0.005, 1e-9, "fp64"), (5000, (0.5, 1.0, 2.0), 3.0, 0.005, 1e-6,
                                                                             "mixed")]:
        b = estimate_bytes(make_params(n, L, a, e, tol=tol, precision=prec))
        assert b > 0


@pytest.mark.parametrize("n,L,a,e,M", [(1000, 1.0, 10.0, 0.01, 0), (20000, 1.0, 20.0, 0.005, 0),
                                       (3000, (0.5, 1.0, 2.0), 3.0, 0.005, 0), (2000, 1.0, 10.0, 0.01, 32)])
def test_resolved_parameters_are_a_fixed_point(n, L, a, e, M):
    """Resolving again with the resolved splitting, cutoff, support and grid
    given explicitly reproduces the instance (the serving path binds requests
    this way, with tables built at submission)."""
    r = resolve(make_params(n, L, a, e, tol=1e-6, M=(M, M, M)))
    r2 = resolve(make_params(n, L, a, e, tol=1e-6, d=r["d"], rc=r["rc"], P=r["P"], M=tuple(r["M"])))
    assert r2 == r


def test_fp64_kernel_tables_match_oracle():
    # the FP64 path's pair kernel (FP64 far series beyond r_mid, closed forms
    # below) vs the oracle's accurate kernel, relative to the largest |H| term
    for a, d, e, rc in [(20, 0.015, 0.005, 0.0707), (10, 0.125, 0.01, 0.6), (3, 0.05, 0.0, 0.25), (45, 0.02, 0.002, 0.1)]:
        r = np.linspace(0, rc, 1201)[1:-1]
        h1, h2 = pb.pair_kernel_tables64(a, d, e, rc, r)
        ex = np.array([oracle.pair_H(rr, a, d, e) for rr in r])
        t1, t2 = np.abs(ex[:, 0]), np.abs(ex[:, 1]) * r * r
        err = (np.abs(h1 - ex[:, 0]) + np.abs(h2 - ex[:, 1]) * r * r) / max(t1.max(), t2.max())
        far = r >= 0.25 * rc
        assert err[far].max() < 1e-11, (a, d, e, err[far].max())
        # closer in: the closed forms of the reference, which cancel as r -> 0
        # when eps = 0 (S - R_d, both singular); with eps > 0 the FP64 series
        # takes over below 0.8 eps
        near = r >= (0.05 * d if e == 0 else 0.0)
        assert err[near].max() < 1e-9, (a, d, e, err[near].max())


def test_kernel_tables_match_oracle():
    # FP32 polynomial tables evaluated as on the GPU vs the FP64 oracle kernel; the
    # last three put alpha delta at 0.001 (closed-form series moments at their
    # smallest), at 5 and 4 (moments by quadrature above alpha delta = 3)
    for a, d, e, rc in [(10, 0.125, 0.01, 0.35), (20, 0.02, 0.005, 0.08), (1, 0.05, 0.005, 0.2), (3, 0.1, 0.0, 0.4),
                        (1, 0.02, 0.001, 0.08), (50, 0.1, 0.02, 0.35), (45, 0.09, 0.0, 0.3)]:
        r = np.linspace(0, rc, 801)[1:-1]
        if e > 0:
            r = np.concatenate([r, e * np.array([0.0, 0.1, 0.5, 0.79, 0.81, 1.0, 2.0, 5.5])])
        h1, h2 = pb.pair_kernel_tables(a, d, e, rc, r)
        ex = np.array([oracle.pair_H(rr, a, d, e) for rr in r])
        if e > 0:
            scale = abs(oracle.pair_H(0.0, a, d, e)[0])
            err = (np.abs(h1 - ex[:, 0]) + np.abs(h2 - ex[:, 1]) * r * r) / scale
            assert err.max() < 1e-6, (a, d, e, err.max())
        else:
            ref = np.abs(ex[:, 0]) + np.abs(ex[:, 1]) * r * r
            err = (np.abs(h1 - ex[:, 0]) + np.abs(h2 - ex[:, 1]) * r * r) / np.maximum(ref, 1 / (8 * np.pi * rc))
            assert err.max() < 2e-6, (a, d, e, err.max())
