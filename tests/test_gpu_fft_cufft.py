"""Side-by-side check of the hand-written FFT passes against cuFFT.

pb_debug_fft_green runs the k-space grid operator of a solve on a device
grid: forward 3D real FFT of the three components (register or shared-memory
Stockham passes), the screened Brinkman Green tensor with Gaussian
deconvolution, and the unnormalised inverse FFT.  The same operator is
built here from torch.fft (cuFFT) in FP64 and compared on random grids:
FP32 grids to 5e-6 and FP64 grids to 1e-12 of the largest output value.
The Green symbol (cuda/periodicBrinkman.h:189-207, cuda/fftBrinkman.h:179-219):
kfac (1 + (1 - e^{-alpha^2 d^2/4}) k^2/alpha^2) e^{-k^2 (d^2/4 - eta/2)}
/ (k^2 (k^2 + alpha^2)) (k^2 I - k k^T), with the Nyquist planes and k = 0
set to zero."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import periodicbrinkman_gb300 as pb  # noqa: E402
from periodicbrinkman_gb300 import _lib  # noqa: E402
from periodicbrinkman_gb300.api import make_params, resolve  # noqa: E402

TOL = {"mixed": 5e-6, "fp64": 1e-12}


def _green_cufft(G, L, M, alpha, d, eta):
    """G: (3, M0, M1, M2) float64 CUDA tensor -> the operator's output, via torch.fft."""
    L = np.asarray(L, dtype=np.float64)
    # the normalisations of spreading and gathering, (pi eta)^{-3/2} each, and h^3 / M^3
    kfac = np.prod(L / np.asarray(M)) / (np.prod(M) * (np.pi * eta) ** 3)
    Gh = torch.fft.rfftn(G, dim=(1, 2, 3), norm="backward")  # unnormalised forward
    dev = G.device
    n0 = torch.fft.fftfreq(M[0], d=1.0 / M[0], dtype=torch.float64, device=dev)
    n1 = torch.fft.fftfreq(M[1], d=1.0 / M[1], dtype=torch.float64, device=dev)
    n2 = torch.arange(M[2] // 2 + 1, dtype=torch.float64, device=dev)
    kx = (2 * np.pi / L[0]) * n0[:, None, None]
    ky = (2 * np.pi / L[1]) * n1[None, :, None]
    kz = (2 * np.pi / L[2]) * n2[None, None, :]
    kn = kx * kx + ky * ky + kz * kz
    a2 = alpha * alpha
    a1oa2 = -np.expm1(-a2 * d * d / 4) / a2
    gexp = d * d / 4 - eta / 2
    zero = (n0[:, None, None] == -M[0] // 2) | (n1[None, :, None] == -M[1] // 2) | (n2[None, None, :] == M[2] // 2)
    zero = zero | (kn == 0)
    knz = torch.where(kn == 0, torch.ones_like(kn), kn)
    s = kfac * (1 + a1oa2 * knz) * torch.exp(-knz * gexp) / (knz * (knz + a2))
    s = torch.where(zero, torch.zeros_like(s), s)
    dr = kx * Gh[0] + ky * Gh[1] + kz * Gh[2]
    out = torch.stack([s * (kn * Gh[0] - kx * dr), s * (kn * Gh[1] - ky * dr), s * (kn * Gh[2] - kz * dr)])
    return torch.fft.irfftn(out, s=tuple(M), dim=(1, 2, 3), norm="forward")  # unnormalised inverse


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
@pytest.mark.parametrize("M,L,alpha,d,P", [
    ((32, 32, 32), (1.0, 1.0, 1.0), 10.0, 0.1, 8),
    ((64, 32, 16), (1.0, 0.5, 0.25), 4.0, 0.05, 8),
    ((128, 128, 128), (1.0, 1.0, 1.0), 20.0, 0.025, 12),
    ((512, 16, 16), (2.0, 0.0625, 0.0625), 30.0, 0.01, 8),
])
def test_fft_green_matches_cufft(prec, M, L, alpha, d, P):
    p = make_params(1000, L, alpha, 0.0, tol=1e-6, d=d, rc=2 * d, M=M, P=P, precision=prec)
    info = resolve(p)
    assert tuple(info["M"]) == tuple(M)
    rng = np.random.default_rng(sum(M))
    G = rng.standard_normal((3,) + tuple(M))
    Gd = torch.from_numpy(G).cuda()
    ref = _green_cufft(Gd, L, M, alpha, info["d"], info["eta"]).cpu().numpy()
    if prec == "mixed":  # M^3 float4 (x, y, z, unused)
        buf = torch.zeros(tuple(M) + (4,), dtype=torch.float32, device="cuda")
        buf[..., :3] = Gd.permute(1, 2, 3, 0).float()
    else:  # four planes of M^3 doubles
        buf = torch.zeros((4,) + tuple(M), dtype=torch.float64, device="cuda")
        buf[:3] = Gd
    torch.cuda.synchronize()
    _lib.check(pb.lib().pb_debug_fft_green(C.byref(p), C.c_void_p(buf.data_ptr()), None))
    got = (buf[..., :3].permute(3, 0, 1, 2) if prec == "mixed" else buf[:3]).double().cpu().numpy()
    if prec == "mixed":  # the FP32 input rounding enters too: compare with the operator of the rounded input
        ref = _green_cufft(Gd.float().double(), L, M, alpha, info["d"], info["eta"]).cpu().numpy()
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err < TOL[prec], err
