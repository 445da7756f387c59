"""The allocation-free entry point pb_fft_brinkman_static against
pb_fft_brinkman, through the C ABI, on two calls in a row.

This file is collected last so that it runs both alone in a fresh process
and after every other test has used the library."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from periodicbrinkman_gb300 import _lib  # noqa: E402

TOL = 1e-13  # relative to max |u|: the two paths differ only in the order of the spreading atomics

_dp, _ip = C.POINTER(C.c_double), C.POINTER(C.c_int)


def _case(seed, n, m, L):
    rng = np.random.default_rng(seed)
    L = np.asarray(L, dtype=np.float64)
    return rng.random((n, 3)) * L, rng.standard_normal((n, 3)), rng.random((m, 3)) * L


def _host_call(y, f, x, L, M, P, msd, e, d, alpha):
    U = np.zeros_like(y)
    Lv, Mv, Pv = (np.ascontiguousarray(L, np.float64), np.ascontiguousarray(M, np.int32),
                  np.ascontiguousarray(P, np.int32))
    _lib.check(_lib.lib().pb_fft_brinkman(U.ctypes.data_as(_dp), y.ctypes.data_as(_dp), y.shape[0],
                                          f.ctypes.data_as(_dp), x.ctypes.data_as(_dp), x.shape[0],
                                          Lv.ctypes.data_as(_dp), Mv.ctypes.data_as(_ip), Pv.ctypes.data_as(_ip),
                                          msd, 0, e, 1e-6, d, alpha))
    return U


def _static_call(y, f, x, L, M, P, msd, e, d, alpha, stream):
    yd, fd, xd = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (y, f, x))
    Ud = torch.full_like(yd, float("nan"))  # every entry must be written
    Lv, Mv, Pv = (np.ascontiguousarray(L, np.float64), np.ascontiguousarray(M, np.int32),
                  np.ascontiguousarray(P, np.int32))
    _lib.check(_lib.lib().pb_fft_brinkman_static(Ud.data_ptr(), yd.data_ptr(), y.shape[0], fd.data_ptr(),
                                                 xd.data_ptr(), x.shape[0], Lv.ctypes.data_as(_dp),
                                                 Mv.ctypes.data_as(_ip), Pv.ctypes.data_as(_ip), msd, e, d, alpha,
                                                 C.c_void_p(stream.cuda_stream)))
    stream.synchronize()
    return Ud.cpu().numpy()


# Against the FP64 oracle's direct k-space sum, max relative error: the
# spectral sum carries the Gaussian window's truncation exp(-(P/2 - 1)^2 / s)
# and aliasing, s = eta / h^2 = P^2 / (2 msd^2): 1e-7 for the reference's
# parameters (P 16, msd 7), 3.7e-6 truncation for P 12, msd 6.
ORACLE_TOL = {41: 1e-7, 42: 2e-5}


def test_static_entry_matches_fft_brinkman_on_two_calls():
    import oracle

    assert torch.cuda.is_available()
    stream = torch.cuda.Stream()
    cases = [
        # seed, n, m, L, M, P, msd, eps, d, alpha
        (41, 3000, 700, [1.0, 1.0, 1.0], [64, 64, 64], [16, 16, 16], 7, 0.01, 0.125, 10.0),
        (42, 1200, 333, [1.0, 0.5, 1.0], [32, 16, 32], [12, 12, 12], 6, 0.0, 0.1, 4.0),
    ]
    for seed, n, m, L, M, P, msd, e, d, a in cases:
        x, f, y = _case(seed, n, m, L)
        ref = _host_call(y, f, x, L, M, P, msd, e, d, a)
        got = _static_call(y, f, x, L, M, P, msd, e, d, a, stream)
        assert np.isfinite(got).all()
        assert np.abs(got - ref).max() <= TOL * np.abs(ref).max(), (seed, np.abs(got - ref).max())
        # and against the FP64 oracle's k-space sum on a subset of the targets
        sel = np.arange(0, m, max(1, m // 40))
        uo = oracle.ewald_velocity(y[sel], x, f, np.asarray(L), a, e, d=d, real=False)
        mx, _ = oracle.rel_errors(got[sel], uo)
        assert mx < ORACLE_TOL[seed], (seed, mx)


def test_static_entry_rejects_sizes_beyond_its_scratch():
    x, f, y = _case(43, 10, 5, [1.0, 1.0, 1.0])
    with pytest.raises(_lib.PbError) as ei:
        _static_call(y, f, x, [1.0, 1.0, 1.0], [128, 128, 128], [16, 16, 16], 7, 0.01, 0.125, 10.0,
                     torch.cuda.Stream())
    assert ei.value.code == _lib.PB_ERR_UNSUPPORTED and "static scratch" in str(ei.value)
    # no autotuned grid: an unset grid or support is refused before anything runs
    for M, P in (([0, 0, 0], [16, 16, 16]), ([64, 0, 64], [16, 16, 16]), ([64, 64, 64], [0, 0, 0])):
        with pytest.raises(_lib.PbError) as ei:
            _static_call(y, f, x, [1.0, 1.0, 1.0], M, P, 7, 0.01, 0.125, 10.0, torch.cuda.Stream())
        assert ei.value.code == _lib.PB_ERR_INVALID
