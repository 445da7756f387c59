"""The dense drop-in against the reference's OWN compiled CUDA kernels on the
GPU: kernelFourier + kernelReal of cuda/periodicBrinkman.h:219-425, built
from the reference's sources into a device-only image by oracle/build_ref.sh
and launched with periodicBrinkman()'s configuration by oracle/ref_launch.cpp.

The reference's kernelFourier leaves out the 1/tau of its host twin (defect
D1: cuda/periodicBrinkman.h:386 against :745), so the drop-in is compared
with tau_scaled = 0 (pb_periodic_brinkman_ex), and with the default 1/tau
scaling where tau = 1.  Both sides converged (real images erfc(M L/d) below
1e-16, wave vectors exp(-(2 pi N/L)^2 d^2/4) below 1e-16)."""
import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import periodicbrinkman_gb300 as pb  # noqa: E402
from periodicbrinkman_gb300 import _lib  # noqa: E402

TOL = 1e-12  # max |A - A_ref| / max |A_ref|

_why = oracle.ref_gpu_available()


def _cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def _dense(m, n):
    return torch.zeros((3 * n, 3 * m), dtype=torch.float64, device="cuda").t()  # column-major (3m, 3n)


def _ours(x, x0, a, d, e, M, N, L, tau_scaled):
    m, n = x.shape[0], x0.shape[0]
    Mx, Nx = pb.shell_counts(L, M, N)
    dA = _dense(m, n)
    Lv = np.ascontiguousarray(np.broadcast_to(np.asarray(L, dtype=np.float64), (3,)))
    Mv, Nv = np.asarray(Mx, dtype=np.int32), np.asarray(Nx, dtype=np.int32)
    import ctypes as C

    xd, x0d = _cuda(x), _cuda(x0)
    _lib.check(pb.lib().pb_periodic_brinkman_ex(dA.data_ptr(), xd.data_ptr(), m, x0d.data_ptr(), n, a, d, e,
                                                 Mv.ctypes.data_as(C.POINTER(C.c_int)),
                                                 Nv.ctypes.data_as(C.POINTER(C.c_int)),
                                                 Lv.ctypes.data_as(C.POINTER(C.c_double)), tau_scaled, None))
    torch.cuda.synchronize()
    return dA.cpu().numpy()


def _reference(x, x0, a, d, e, M, N, L):
    m, n = x.shape[0], x0.shape[0]
    dA = _dense(m, n)
    xd, x0d = _cuda(x), _cuda(x0)
    torch.cuda.synchronize()
    oracle.ref_gpu_periodic_brinkman(dA.data_ptr(), xd.data_ptr(), m, x0d.data_ptr(), n, a, d, e, M, N, L)
    return dA.cpu().numpy()


@pytest.mark.skipif(_why is not None, reason=str(_why))
@pytest.mark.parametrize("case", [
    # m, n, L, alpha, d, eps, M (real shells), N (Fourier shells), seed
    ("iso_config1_params", 40, 56, (1.0, 1.0, 1.0), 10.0, 0.125, 0.01, 1, 16, 1),
    ("iso_singular", 24, 40, (1.0, 1.0, 1.0), 4.0, 0.2, 0.0, 2, 10, 2),
    ("aniso_no_tau", 32, 48, (1.0, 0.8, 1.25), 7.0, 0.15, 0.02, 2, 14, 3),
])
def test_dense_drop_in_matches_reference_cuda_build(case):
    name, m, n, L, a, d, e, M, N, seed = case
    rng = np.random.default_rng(seed)
    Lv = np.asarray(L)
    x, x0 = rng.random((m, 3)) * Lv, rng.random((n, 3)) * Lv
    x0[:5] = x[:5]  # coincident target/source pairs: the r -> 0 limits on both sides
    ref = _reference(x, x0, a, d, e, M, N, L)
    assert np.isfinite(ref).all() and np.abs(ref).max() > 0
    got = _ours(x, x0, a, d, e, M, N, L, tau_scaled=0)
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err <= TOL, (name, err)
    if np.prod(Lv) == 1.0:  # tau = 1: the default (1/tau-scaled) drop-in is the same sum
        dA = _dense(m, n)
        pb.periodicBrinkman(dA, _cuda(x), _cuda(x0), a, d, e, M, N, L)
        err1 = np.abs(dA.cpu().numpy() - ref).max() / np.abs(ref).max()
        assert err1 <= TOL, (name, err1)


@pytest.mark.skipif(_why is not None, reason=str(_why))
def test_reference_cuda_build_accumulates():
    """The reference's kernels add into dA (dA +=, cuda/periodicBrinkman.h:304, 415) as the drop-in does."""
    rng = np.random.default_rng(9)
    x, x0 = rng.random((8, 3)), rng.random((12, 3))
    once = _reference(x, x0, 5.0, 0.2, 0.01, 1, 8, (1.0, 1.0, 1.0))
    dA = _dense(8, 12)
    xd, x0d = _cuda(x), _cuda(x0)
    torch.cuda.synchronize()
    for _ in range(2):
        oracle.ref_gpu_periodic_brinkman(dA.data_ptr(), xd.data_ptr(), 8, x0d.data_ptr(), 12, 5.0, 0.2, 0.01, 1, 8,
                                         (1.0, 1.0, 1.0))
    assert np.abs(dA.cpu().numpy() - 2 * once).max() <= 1e-13 * np.abs(once).max()
