"""FP64 CPU oracle for the periodic regularized Brinkman hot path.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this package, and only as the checker
(or, for ``bench.py --impl reference``, as the timed CPU restatement of the
reference's algorithm).  The product library never imports it.

The C sources (``pb_oracle.c``) restate the reference's algorithm in double
precision; see the header of that file for the reference file:line each part
follows.  ``ref_lib()`` loads the reference's own host code compiled from its
sources by ``build_ref.sh`` (present only where the reference tree exists; it
is used to generate the golden fixtures under ``tests/golden/``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "libpb_oracle.so")
_REF_PATH = os.path.join(_HERE, "_ref", "libpbref.so")

REAL, KSPACE, ZERO_MODE = 1, 2, 4

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lib = None


def build(force: bool = False) -> str:
    """Compile pb_oracle.c into oracle/_build/libpb_oracle.so (gcc, OpenMP)."""
    src = os.path.join(_HERE, "pb_oracle.c")
    if not force and os.path.exists(_LIB_PATH) and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(src):
        return _LIB_PATH
    os.makedirs(_BUILD, exist_ok=True)
    tmp = _LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off", "-o", tmp, src, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def build_ref() -> bool:
    """Build oracle/_ref/libpbref.so from the reference sources if they exist here."""
    script = os.path.join(_HERE, "build_ref.sh")
    subprocess.run(["bash", script], check=True)
    return os.path.exists(_REF_PATH)


_REF_LAUNCH_SRC = os.path.join(_HERE, "ref_launch.cpp")
_REF_LAUNCH_LIB = os.path.join(_BUILD, "libpbref_launch.so")
_REF_IMAGES = [os.path.join(_HERE, "_ref", "ref_kernels." + k) for k in ("cubin", "ptx")]
_ref_gpu = None


def ref_gpu_available() -> str | None:
    """None when the reference's compiled kernel image is present here, else why not."""
    if not any(os.path.exists(p) for p in _REF_IMAGES):
        return ("the reference's kernel image oracle/_ref/ref_kernels.{cubin,ptx} was not built (it needs the "
                "reference's sources, which stay out of this repository)")
    return None


def ref_gpu():
    """The launcher of the reference's own CUDA kernels (ref_launch.cpp), built
    here with g++ against the CUDA driver API, with the kernel image loaded
    into the current CUDA context.  TEST INFRASTRUCTURE: the checker of the
    dense drop-in and a timed baseline, never the product path."""
    global _ref_gpu
    if _ref_gpu is not None:
        return _ref_gpu
    why = ref_gpu_available()
    if why:
        raise RuntimeError(why)
    if not os.path.exists(_REF_LAUNCH_LIB) or os.path.getmtime(_REF_LAUNCH_LIB) < os.path.getmtime(_REF_LAUNCH_SRC):
        os.makedirs(_BUILD, exist_ok=True)
        tmp = _REF_LAUNCH_LIB + f".tmp{os.getpid()}"
        cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
        subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I", os.path.join(cuda, "include"), "-o", tmp,
                        _REF_LAUNCH_SRC, "-L", os.path.join(cuda, "lib64", "stubs"), "-lcuda"], check=True)
        os.replace(tmp, _REF_LAUNCH_LIB)
    L = C.CDLL(_REF_LAUNCH_LIB)
    L.refk_error.restype = C.c_char_p
    L.refk_load.argtypes = [C.c_char_p]
    L.refk_periodic_brinkman.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_double,
                                         C.c_double, C.c_double, C.c_int, C.c_int, _dp, C.c_int]
    errs = []
    for img in _REF_IMAGES:
        if os.path.exists(img):
            if L.refk_load(img.encode()) == 0:
                _ref_gpu = L
                return L
            errs.append(f"{os.path.basename(img)}: {L.refk_error().decode()}")
    raise RuntimeError("reference kernel image not loaded: " + "; ".join(errs))


def ref_gpu_periodic_brinkman(dA_ptr, dx_ptr, m, dx0_ptr, n, a, d, e, M, N, L, max_block=256):
    """The reference's periodicBrinkman() on its own compiled kernels: dA
    (device, 3m x 3n column-major) += A.  Device pointers; waits."""
    Lv = np.ascontiguousarray(np.broadcast_to(np.asarray(L, dtype=np.float64), (3,)))
    lib_ = ref_gpu()
    rc = lib_.refk_periodic_brinkman(dA_ptr, dx_ptr, int(m), dx0_ptr, int(n), float(a), float(d), float(e), int(M),
                                     int(N), _p(Lv), int(max_block))
    if rc != 0:
        raise RuntimeError("reference kernels: " + lib_.refk_error().decode())


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        L = _lib
        L.pbo_experf.restype = C.c_double
        L.pbo_experf.argtypes = [C.c_double] * 3
        for name in ("pbo_diffH", "pbo_regH"):
            getattr(L, name).argtypes = [C.c_double] * 3 + [_dp, _dp]
        L.pbo_singH.argtypes = [C.c_double, C.c_double, _dp, _dp]
        L.pbo_vR.argtypes = [_dp, _dp, C.c_double, C.c_double, C.c_double]
        L.pbo_vF.argtypes = [_dp, _dp, C.c_double, C.c_double, _dp]
        L.pbo_pairH.argtypes = [C.c_double] * 4 + [_dp, _dp]
        L.pbo_reg_quad.argtypes = [C.c_double] * 4 + [C.c_int, _dp, _dp]
        L.pbo_shell_counts.argtypes = [_dp, C.c_int, C.c_int, _ip, _ip]
        L.pbo_shell_matrix.argtypes = [_dp, _dp, C.c_int, _dp, C.c_int, C.c_double, C.c_double,
                                       C.c_double, _ip, _ip, _dp]
        L.pbo_ewald_velocity.restype = C.c_int
        L.pbo_ewald_velocity.argtypes = [_dp, _dp, C.c_int, _dp, _dp, C.c_int, _dp] + [C.c_double] * 5 + [C.c_int]
        L.pbo_set_eps_switch.argtypes = [C.c_double]
        L.pbo_get_eps_switch.restype = C.c_double
        L.pbo_phihat.restype = C.c_double
        L.pbo_phihat.argtypes = [C.c_double] * 3
        L.pbo_brinkmanlet.argtypes = [_dp, _dp, C.c_double, C.c_double]
        L.pbo_brinkmanlet_velocity.argtypes = [_dp, _dp, C.c_int, _dp, _dp, C.c_int, C.c_double, C.c_double]
        L.pbo_num_threads.restype = C.c_int
        L.pbo_set_num_threads.argtypes = [C.c_int]
    return _lib


def ref_lib():
    """The reference's own host code (only where oracle/_ref was built)."""
    if not os.path.exists(_REF_PATH):
        return None
    R = C.CDLL(_REF_PATH)
    for name in ("ref_diffH", "ref_regH"):
        getattr(R, name).argtypes = [C.c_double] * 3 + [_dp]
    R.ref_singH.argtypes = [C.c_double, C.c_double, _dp]
    R.ref_experf.restype = C.c_double
    R.ref_experf.argtypes = [C.c_double] * 3
    R.ref_vR.argtypes = [_dp, _dp, C.c_double, C.c_double, C.c_double]
    R.ref_vF.argtypes = [_dp, _dp, C.c_double, C.c_double, _dp]
    R.ref_shells.argtypes = [_dp, _dp, C.c_int, _dp, C.c_int, _ip, _ip, _dp, C.c_double, C.c_double, C.c_double]
    return R


def _p(a):
    return a.ctypes.data_as(_dp)


def _c64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def set_threads(n: int) -> None:
    lib().pbo_set_num_threads(int(n))


def num_threads() -> int:
    return int(lib().pbo_num_threads())


def diffH(r2: float, a: float, d: float):
    h1, h2 = C.c_double(), C.c_double()
    lib().pbo_diffH(r2, a, d, C.byref(h1), C.byref(h2))
    return h1.value, h2.value


def regH(r2: float, a: float, d: float):
    h1, h2 = C.c_double(), C.c_double()
    lib().pbo_regH(r2, a, d, C.byref(h1), C.byref(h2))
    return h1.value, h2.value


def pair_H(r: float, a: float, d: float, e: float):
    """Accurate real-space kernel (R_e - R_d, or S - R_d for e = 0)."""
    h1, h2 = C.c_double(), C.c_double()
    lib().pbo_pairH(r, a, d, e, C.byref(h1), C.byref(h2))
    return h1.value, h2.value


def reg_quad(r: float, a: float, d1: float, d2: float = 0.0, diff: bool = False):
    h1, h2 = C.c_double(), C.c_double()
    lib().pbo_reg_quad(r, a, d1, d2 if diff else d1, 1 if diff else 0, C.byref(h1), C.byref(h2))
    return h1.value, h2.value


def vR(xh, a, d, e):
    A = np.zeros(9)
    lib().pbo_vR(_p(A), _p(_c64(xh)), a, d, e)
    return A.reshape(3, 3, order="F")


def vF(xh, a, d, k):
    A = np.zeros(9)
    lib().pbo_vF(_p(A), _p(_c64(xh)), a, d, _p(_c64(k)))
    return A.reshape(3, 3, order="F")


def shell_counts(L, M: int, N: int):
    """Per-axis real/Fourier shell counts of periodicBrinkman (P.h:457-487)."""
    Mx = np.zeros(3, np.int32)
    Nx = np.zeros(3, np.int32)
    lib().pbo_shell_counts(_p(_c64(L)), int(M), int(N), Mx.ctypes.data_as(_ip), Nx.ctypes.data_as(_ip))
    return Mx, Nx


def shell_matrix(x, x0, a, d, e, Mx, Nx, L):
    """Dense 3m x 3n mobility matrix by real and Fourier shells (with 1/tau)."""
    x = _c64(x)
    x0 = _c64(x0)
    m, n = x.shape[0], x0.shape[0]
    A = np.zeros(9 * m * n)
    Mx = np.ascontiguousarray(Mx, np.int32)
    Nx = np.ascontiguousarray(Nx, np.int32)
    lib().pbo_shell_matrix(_p(A), _p(x), m, _p(x0), n, a, d, e, Mx.ctypes.data_as(_ip), Nx.ctypes.data_as(_ip),
                           _p(_c64(L)))
    return A.reshape(3 * m, 3 * n, order="F")


def choose_split(n: int, m: int, L) -> float:
    """Splitting blob width that balances the oracle's real and k-space cost.

    The total is independent of this choice; it only sets the oracle's run
    time (real space ~ m*n*(6d)^3/tau closed-form pairs, k space ~
    (n+m)*tau/d^3 structure-factor terms)."""
    L = np.broadcast_to(np.asarray(L, dtype=np.float64), (3,))
    tau = float(np.prod(L))
    c_r, c_k = 60e-9, 1.5e-9
    real_coef = m * n * (4 * np.pi / 3) * 216.0 / tau * c_r
    k_coef = (n + m) * (2 * np.pi / 3) * (14.0 / (2 * np.pi)) ** 3 * tau * c_k
    d = (k_coef / real_coef) ** (1.0 / 6.0)
    return float(min(max(d, 1e-4), 0.5 * float(L.min()) * 4))


def ewald_velocity(y, x, f, L, alpha, eps, d=None, rc=0.0, kc=0.0, real=True, kspace=True, zero_mode=False):
    """Converged FP64 direct-Ewald velocities at targets y (m x 3).

    Sources x (n x 3) carry forces f (n x 3) in the periodic box L.  The
    k = 0 mode is dropped unless zero_mode (then u += sum f / (alpha^2 tau))."""
    y = _c64(y).reshape(-1, 3)
    x = _c64(x).reshape(-1, 3)
    f = _c64(f).reshape(-1, 3)
    m, n = y.shape[0], x.shape[0]
    if d is None:
        d = choose_split(n, m, L)
    U = np.zeros((m, 3))
    flags = (REAL if real else 0) | (KSPACE if kspace else 0) | (ZERO_MODE if zero_mode else 0)
    Lv = np.ascontiguousarray(np.broadcast_to(np.asarray(L, dtype=np.float64), (3,)))
    rcode = lib().pbo_ewald_velocity(_p(U), _p(y), m, _p(x), _p(f), n, _p(Lv), float(alpha), float(eps),
                                     float(d), float(rc), float(kc), flags)
    if rcode != 0:
        raise ValueError("oracle: bad input")
    return U


def brinkmanlet(xh, alpha, d):
    """The reference's Brinkmanlet tensor (3x3) at displacement xh (faithful closed forms)."""
    A = np.zeros(9)
    xv = _c64(xh).reshape(3)
    lib().pbo_brinkmanlet(_p(A), _p(xv), float(alpha), float(d))
    return A.reshape(3, 3).T  # column-major storage -> (row, col)


def brinkmanlet_velocity(y, x, f, alpha, eps):
    """Free-space (non-periodic) velocities at y of forces f at x, accurate FP64 kernel."""
    y = _c64(y).reshape(-1, 3)
    x = _c64(x).reshape(-1, 3)
    f = _c64(f).reshape(-1, 3)
    U = np.zeros_like(y)
    lib().pbo_brinkmanlet_velocity(_p(U), _p(y), y.shape[0], _p(x), _p(f), x.shape[0], float(alpha), float(eps))
    return U


def rel_errors(u, u_ref):
    """(max, rms) relative velocity error: max_i |u_i - u*_i| / max_i |u*_i|
    and ||u - u*||_2 / ||u*||_2."""
    u = np.asarray(u, dtype=np.float64).reshape(-1, 3)
    u_ref = np.asarray(u_ref, dtype=np.float64).reshape(-1, 3)
    nrm = np.linalg.norm(u_ref, axis=1).max()
    mx = np.linalg.norm(u - u_ref, axis=1).max() / nrm
    rms = np.linalg.norm(u - u_ref) / np.linalg.norm(u_ref)
    return float(mx), float(rms)
