"""GPU: strongly clustered inputs (Gaussian clusters much smaller than the
box, the shape of the clustered configuration): crowded cells (beyond the
cell sort's rank limit), many pairs inside r_mid per chunk (the near queue's
overflow path) and long cell rows, against the FP64 path and the oracle."""
import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import periodicbrinkman_gb300 as pb  # noqa: E402


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


@pytest.fixture(scope="module", autouse=True)
def _device():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _clusters(n, ncl, sigma, L, seed):
    rng = np.random.default_rng(seed)
    centres = rng.random((ncl, 3)) * L
    x = (centres[rng.integers(0, ncl, n)] + sigma * rng.standard_normal((n, 3))) % L
    f = rng.standard_normal((n, 3))
    return x, f, rng


@pytest.mark.parametrize("n,ncl,sigma", [(20000, 20, 0.02), (12000, 3, 0.01)])
def test_clustered_sources_match_fp64_and_oracle(n, ncl, sigma):
    L, alpha, eps = 2.0, 5.0, 0.002
    x, f, rng = _clusters(n, ncl, sigma, L, 3000 + ncl)
    u64 = pb.solve(cuda(x), cuda(f), L, alpha, eps, tol=1e-6, precision="fp64").cpu().numpy()
    umx = pb.solve(cuda(x), cuda(f), L, alpha, eps, tol=1e-6, precision="mixed").cpu().numpy()
    assert np.isfinite(umx).all()
    # the mixed path against the FP64 path over every target (max-norm relative error)
    assert oracle.rel_errors(umx, u64)[0] < 1e-6
    idx = rng.choice(n, 24, replace=False)
    ref = oracle.ewald_velocity(x[idx], x, f, L, alpha, eps)
    assert oracle.rel_errors(umx[idx], ref)[0] < 1e-6


def test_clustered_targets_apart_from_sources():
    L, alpha, eps = 2.0, 5.0, 0.002
    x, f, rng = _clusters(15000, 10, 0.02, L, 3100)
    y, _, _ = _clusters(6000, 10, 0.02, L, 3100)  # the same cluster centres
    u64 = pb.solve(cuda(x), cuda(f), L, alpha, eps, y=cuda(y), tol=1e-6, precision="fp64").cpu().numpy()
    umx = pb.solve(cuda(x), cuda(f), L, alpha, eps, y=cuda(y), tol=1e-6, precision="mixed").cpu().numpy()
    assert oracle.rel_errors(umx, u64)[0] < 1e-6
