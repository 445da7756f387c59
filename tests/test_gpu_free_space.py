"""GPU free-space Brinkmanlet (the reference's Brinkmanlet(),
cuda/periodicBrinkman.h:119-141) against the FP64 oracle: velocities with
the accurate kernel (Fourier integral of the blob below 0.2 eps), and the
dense tensor form against the oracle's faithful restatement of the
reference's closed forms."""
import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import periodicbrinkman_gb300 as pb  # noqa: E402


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


@pytest.mark.parametrize("alpha,eps", [(10.0, 0.01), (1.0, 0.005), (40.0, 0.05), (5.0, 0.0), (0.5, 0.0)])
def test_free_space_velocity_matches_oracle(alpha, eps):
    rng = np.random.default_rng(int(alpha * 100 + eps * 1e4))
    n, m = 700, 300
    x = rng.random((n, 3))
    f = rng.standard_normal((n, 3))
    y = rng.random((m, 3))
    y[:20] = x[:20]  # coincident pairs: R_eps(0) (eps > 0), skipped (eps = 0)
    y[20:40] = x[20:40] + 1e-4 * rng.standard_normal((20, 3))  # r << eps: the series
    ref = oracle.brinkmanlet_velocity(y, x, f, alpha, eps)
    for host in (True, False):
        u = pb.Brinkmanlet(y, x, f, alpha, eps) if host else \
            pb.Brinkmanlet(cuda(y), cuda(x), cuda(f), alpha, eps).cpu().numpy()
        mx, rms = oracle.rel_errors(u, ref)
        assert mx < 1e-10 and rms < 1e-10, (host, mx, rms)


@pytest.mark.parametrize("eps", [0.02, 0.0])
def test_free_space_matrix_matches_reference_tensor(eps):
    rng = np.random.default_rng(7)
    m, n, alpha = 9, 13, 6.0
    dx, dx0 = rng.random((m, 3)), rng.random((n, 3))
    dA = torch.full((3 * n, 3 * m), 0.25, dtype=torch.float64, device="cuda").t()
    pb.brinkmanlet_matrix(dA, cuda(dx), cuda(dx0), alpha, eps)
    A = dA.cpu().numpy() - 0.25  # accumulated
    for i in range(m):
        for j in range(n):
            T = oracle.brinkmanlet(dx[i] - dx0[j], alpha, eps)
            blk = A[3 * i:3 * i + 3, 3 * j:3 * j + 3]
            assert np.abs(blk - T).max() <= 1e-12 * max(1.0, np.abs(T).max()), (i, j)


def test_free_space_rejects_bad_input():
    x = np.zeros((3, 3))
    with pytest.raises(pb.PbError):
        pb.Brinkmanlet(x, x, x, -1.0, 0.01)
    bad = x.copy()
    bad[1, 1] = np.nan
    with pytest.raises(pb.PbError):
        pb.Brinkmanlet(x, bad, x, 1.0, 0.01)
