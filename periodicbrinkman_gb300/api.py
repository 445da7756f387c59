"""Host-side mirror of the reference's entry points over the C ABI.

Host buffers are numpy float64 arrays, device buffers are torch CUDA float64
tensors; a "3 x N column-major matrix" of the reference is an (N, 3) array.
"""
from __future__ import annotations

import ctypes as C
from typing import Iterable, Sequence

import numpy as np

from ._lib import (
    PB_DEVICE,
    PB_HOST,
    PB_OK,
    PB_PREC_FP64,
    PB_PREC_MIXED,
    InstanceInfo,
    PbError,
    ServerConfig,
    ServerCounters,
    SlotConfig,
    SolveParams,
    TuneRow,
    check,
    lib,
)

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def _is_torch(a) -> bool:
    return type(a).__module__.startswith("torch")


def _where(arrs) -> int:
    dev = [_is_torch(a) and a.is_cuda for a in arrs if a is not None]
    if all(dev):
        return PB_DEVICE
    if not any(dev):
        return PB_HOST
    raise ValueError("mix of host and device buffers")


def _ptr(a) -> int | None:
    if a is None:
        return None
    if _is_torch(a):
        if a.dtype.__str__() != "torch.float64" or not a.is_contiguous():
            raise ValueError("device buffers must be contiguous float64 tensors")
        return a.data_ptr()
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise ValueError("host buffers must be C-contiguous float64 arrays")
    return a.ctypes.data


def make_params(n_src: int, L, alpha: float, eps: float, n_tgt: int = 0, tol: float = 0.0, d: float = 0.0,
                rc: float = 0.0, M=(0, 0, 0), P: int = 0, m_std: float = 0.0, precision: str | int = "mixed",
                flags: int = 0) -> SolveParams:
    p = SolveParams()
    p.n_src = int(n_src)
    p.n_tgt = int(n_tgt)
    Lv = np.broadcast_to(np.asarray(L, dtype=np.float64), (3,))
    Mv = np.broadcast_to(np.asarray(M, dtype=np.int64), (3,))
    for a in range(3):
        p.L[a] = float(Lv[a])
        p.M[a] = int(Mv[a])
    p.alpha = float(alpha)
    p.eps = float(eps)
    p.tol = float(tol)
    p.d = float(d)
    p.rc = float(rc)
    p.P = int(P)
    p.m_std = float(m_std)
    if isinstance(precision, str):
        precision = {"mixed": PB_PREC_MIXED, "fp64": PB_PREC_FP64}[precision]
    p.precision = int(precision)
    p.flags = int(flags)
    return p


class Plan:
    """Device buffers, tables and a CUDA graph for a batch of instances."""

    def __init__(self, params: SolveParams | Sequence[SolveParams]):
        if isinstance(params, SolveParams):
            params = [params]
        self.params = list(params)
        arr = (SolveParams * len(self.params))(*self.params)
        h = C.c_void_p()
        check(lib().pb_plan_create(arr, len(self.params), C.byref(h)))
        self._h = h
        self.n_src = sum(p.n_src for p in self.params)
        self.n_tgt = sum(p.n_tgt if p.n_tgt > 0 else p.n_src for p in self.params)
        self.n_y = sum(p.n_tgt for p in self.params)

    def execute(self, x, f, y=None, U=None, stream=None):
        """Packed inputs of all instances; returns U (n_tgt_total, 3)."""
        if U is None:
            if _is_torch(x):
                import torch

                U = torch.empty((self.n_tgt, 3), dtype=torch.float64, device=x.device)
            else:
                U = np.empty((self.n_tgt, 3))
        where = _where([x, f, y, U])
        s = None
        if stream is not None:
            s = stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)
        check(lib().pb_plan_execute(self._h, _ptr(x), _ptr(f), _ptr(y), _ptr(U), where, s))
        return U

    def execute_forces(self, f, U=None, stream=None):
        """New forces at the positions of the last `execute` (a matrix-free
        mobility product: the cell lists and work items are reused)."""
        if U is None:
            if _is_torch(f):
                import torch

                U = torch.empty((self.n_tgt, 3), dtype=torch.float64, device=f.device)
            else:
                U = np.empty((self.n_tgt, 3))
        where = _where([f, U])
        s = None
        if stream is not None:
            s = stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)
        check(lib().pb_plan_execute_forces(self._h, _ptr(f), _ptr(U), where, s))
        return U

    def status(self) -> None:
        """Waits for the last execution and raises PbError if the device found a
        non-finite input or a capacity overflow (pb_plan_status)."""
        check(lib().pb_plan_status(self._h))

    def set_item_capacity(self, cap: int) -> None:
        """Testing aid: lower the real-space work-item capacity."""
        check(lib().pb_plan_set_item_capacity(self._h, int(cap)))

    def info(self, i: int = 0) -> dict:
        inf = InstanceInfo()
        check(lib().pb_plan_instance_info(self._h, i, C.byref(inf)))
        return {"d": inf.d, "rc": inf.rc, "eta": inf.eta, "m_std": inf.m_std, "M": list(inf.M), "P": inf.P,
                "ncell": list(inf.ncell), "npoly": inf.npoly, "pairs_est": int(inf.pairs_est)}

    @property
    def device_bytes(self) -> int:
        return int(lib().pb_plan_device_bytes(self._h))

    @property
    def kernel_count(self) -> int:
        return int(lib().pb_plan_kernel_count(self._h))

    def set_timing(self, on: bool = True) -> None:
        check(lib().pb_plan_set_timing(self._h, 1 if on else 0))

    def stage_ms(self) -> list[float]:
        out = np.zeros(6)
        check(lib().pb_plan_stage_ms(self._h, out.ctypes.data_as(_dp)))
        return out.tolist()

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().pb_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def make_slot(M: int, max_instances: int, max_src: int, max_tgt: int, max_cells: int = 1 << 20,
              precision: str | int = "mixed", npoly: int = 18) -> "Plan":
    """A capacity plan (serving slot) for instances on an M^3 grid."""
    c = SlotConfig()
    for a in range(3):
        c.M[a] = int(M)
    c.max_instances, c.max_src, c.max_tgt, c.max_cells = int(max_instances), int(max_src), int(max_tgt), int(max_cells)
    c.precision = {"mixed": PB_PREC_MIXED, "fp64": PB_PREC_FP64}.get(precision, precision)
    c.npoly = int(npoly)
    h = C.c_void_p()
    check(lib().pb_plan_create_slot(C.byref(c), C.byref(h)))
    plan = Plan.__new__(Plan)
    plan._h = h
    plan.params = []
    plan.n_src = plan.n_tgt = plan.n_y = 0
    return plan


def slot_estimate_bytes(M: int, max_instances: int, max_src: int, max_tgt: int, max_cells: int,
                        precision: str | int = "mixed", npoly: int = 18) -> int:
    """Device bytes of a capacity plan (pb_slot_estimate_bytes), host only."""
    c = SlotConfig()
    for a in range(3):
        c.M[a] = int(M)
    c.max_instances, c.max_src, c.max_tgt, c.max_cells = int(max_instances), int(max_src), int(max_tgt), int(max_cells)
    c.precision = {"mixed": PB_PREC_MIXED, "fp64": PB_PREC_FP64}.get(precision, precision)
    c.npoly = int(npoly)
    v = int(lib().pb_slot_estimate_bytes(C.byref(c)))
    if v < 0:
        check(v)
    return v


def bind(plan: "Plan", params) -> None:
    """Bind instances to a plan (see pb_plan_bind); sets the packed sizes."""
    params = list(params)
    arr = (SolveParams * max(len(params), 1))(*params)
    check(lib().pb_plan_bind(plan._h, arr, len(params)))
    plan.params = params
    plan.n_src = sum(p.n_src for p in params)
    plan.n_tgt = sum(p.n_tgt if p.n_tgt > 0 else p.n_src for p in params)
    plan.n_y = sum(p.n_tgt for p in params)


class Server:
    """Continuous-batching server (pb_server_*): submit host requests, wait."""

    def __init__(self, precision: str | int = "mixed", budget_bytes: int = 150 << 30, max_batch: int = 4,
                 slots_per_grid: int = 4, grids=(8, 16, 32, 64, 128, 256), max_src: int = 1 << 18,
                 max_tgt: int = 0, queue_capacity: int = 0, linger_us: int = 0, max_dynamic_per_grid: int = 0,
                 dynamic_idle_ms: int = 0):
        c = ServerConfig()
        c.budget_bytes = int(budget_bytes)
        c.precision = {"mixed": PB_PREC_MIXED, "fp64": PB_PREC_FP64}.get(precision, precision)
        c.max_batch = int(max_batch)
        c.slots_per_grid = int(slots_per_grid)
        c.n_grids = len(grids)
        for i, g in enumerate(grids):
            c.grids[i] = int(g)
        c.max_src = int(max_src)
        c.max_tgt = int(max_tgt)
        c.queue_capacity = int(queue_capacity)
        c.linger_us = int(linger_us)
        c.max_dynamic_per_grid = int(max_dynamic_per_grid)
        c.dynamic_idle_ms = int(dynamic_idle_ms)
        self.precision = c.precision
        h = C.c_void_p()
        check(lib().pb_server_create(C.byref(c), C.byref(h)))
        self._h = h
        self._live = {}

    def submit(self, x, f, L, alpha, eps, y=None, out=None, **kw) -> int:
        """Queue one solve; returns a ticket.  Buffers are kept until done.

        `out` (optional): a C-contiguous float64 (targets, 3) array for the
        velocities.  Page-locked inputs and `out` (e.g. numpy views of
        torch pin_memory tensors) are copied by DMA without host staging."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        f = np.ascontiguousarray(f, dtype=np.float64)
        y = None if y is None else np.ascontiguousarray(y, dtype=np.float64)
        m = 0 if y is None else y.shape[0]
        p = make_params(x.shape[0], L, alpha, eps, n_tgt=m, precision=self.precision, **kw)
        if out is None:
            U = np.empty((m if m else x.shape[0], 3))
        else:
            U = out
            if U.dtype != np.float64 or not U.flags.c_contiguous or U.shape != (m if m else x.shape[0], 3):
                raise ValueError("out must be a C-contiguous float64 (targets, 3) array")
        t = C.c_longlong()
        check(lib().pb_server_submit(self._h, C.byref(p), x.ctypes.data, f.ctypes.data,
                                     None if y is None else y.ctypes.data, U.ctypes.data, C.byref(t)))
        self._live[t.value] = (x, f, y, U)
        return t.value

    def poll(self, ticket: int):
        st, status, lat = C.c_int(), C.c_int(), C.c_double()
        check(lib().pb_server_poll(self._h, ticket, C.byref(st), C.byref(status), C.byref(lat)))
        return st.value, status.value, lat.value

    def result(self, ticket: int, timeout: float = 60.0):
        """Wait for a request; returns (U, latency_s) and forgets it."""
        status, lat = C.c_int(), C.c_double()
        check(lib().pb_server_wait(self._h, ticket, float(timeout), C.byref(status), C.byref(lat)))
        U = self._live.pop(ticket)[3]
        lib().pb_server_release(self._h, ticket)
        if status.value != PB_OK:
            raise PbError(status.value, f"request {ticket} failed")
        return U, lat.value

    def drain(self, timeout: float = 600.0) -> None:
        check(lib().pb_server_drain(self._h, float(timeout)))

    def stats(self) -> dict:
        c = ServerCounters()
        check(lib().pb_server_stats(self._h, C.byref(c)))
        return {k: getattr(c, k) for k, _ in c._fields_}

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().pb_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def resolve(params: SolveParams) -> dict:
    """The autotuner's resolved parameters for one instance (host only)."""
    inf = InstanceInfo()
    check(lib().pb_resolve(C.byref(params), C.byref(inf)))
    return {"d": inf.d, "rc": inf.rc, "eta": inf.eta, "m_std": inf.m_std, "M": list(inf.M), "P": inf.P,
            "ncell": list(inf.ncell), "npoly": inf.npoly, "pairs_est": int(inf.pairs_est)}


def tune_report(x, f, L, alpha, eps, y=None, d_values=(0.0,), ref_tol: float = 0.0, **kw) -> list[dict]:
    """pb_tune_report: per candidate splitting width (0 = autotuned) the
    resolved (d, rc, M, P), the max / RMS relative error against the FP64
    reference solution at ref_tol (0 = 1e-12), and the device time (ms)."""
    n = int(x.shape[0])
    m = int(y.shape[0]) if y is not None else 0
    p = make_params(n, L, alpha, eps, n_tgt=m, **kw)
    where = _where([x, f, y])
    dv = np.ascontiguousarray(d_values, dtype=np.float64)
    rows = (TuneRow * max(len(dv), 1))()
    check(lib().pb_tune_report(C.byref(p), _ptr(x), _ptr(f), _ptr(y), where, dv.ctypes.data_as(_dp), len(dv),
                               float(ref_tol), rows))
    return [{"status": r.status, "d": r.d, "rc": r.rc, "M": list(r.M), "P": r.P, "pairs_est": int(r.pairs_est),
             "max_err": r.max_err, "rms_err": r.rms_err, "ms": r.ms} for r in rows[:len(dv)]]


def estimate_bytes(params: SolveParams | Iterable[SolveParams]) -> int:
    if isinstance(params, SolveParams):
        params = [params]
    params = list(params)
    arr = (SolveParams * len(params))(*params)
    v = int(lib().pb_plan_estimate_bytes(arr, len(params)))
    if v < 0:
        check(v)
    return v


def solve(x, f, L, alpha, eps, y=None, **kw):
    """Velocities (m, 3) at targets y (default: the sources x) of forces f at x."""
    n = int(x.shape[0])
    m = int(y.shape[0]) if y is not None else 0
    p = make_params(n, L, alpha, eps, n_tgt=m, **kw)
    with Plan(p) as plan:
        U = plan.execute(x, f, y)
        plan.status()
    return U


def periodicBrinkman(dA, dx, dx0, a, d, e, M, N, L, maxBlockSize: int = 256):
    """Mirror of periodicBrinkman (cuda/periodicBrinkman.h:432-441).

    dA: torch CUDA float64 (3m, 3n) in column-major storage (dA.t() contiguous),
    accumulated into.  dx: (m, 3), dx0: (n, 3) CUDA float64 (3 x m / 3 x n
    column-major).  L: 3 host numbers."""
    if not (_is_torch(dA) and dA.is_cuda):
        raise ValueError("periodicBrinkman works on device tensors")
    m, n = int(dx.shape[0]), int(dx0.shape[0])
    if tuple(dA.shape) != (3 * m, 3 * n) or not dA.t().is_contiguous():
        raise ValueError("dA must be (3m, 3n) column-major")
    Lv = np.ascontiguousarray(np.broadcast_to(np.asarray(L, dtype=np.float64), (3,)))
    check(lib().pb_periodic_brinkman(dA.data_ptr(), _ptr(dx), m, _ptr(dx0), n, float(a), float(d), float(e), int(M),
                                     int(N), Lv.ctypes.data_as(_dp), int(maxBlockSize)))
    return dA


def fftBrinkman(U, y, f, xn, L, M, P, m, C_, e, tol, d, alpha=1.0):
    """Mirror of fftBrinkman (cuda/fftBrinkman.h:34-50): k-space velocities.

    Host numpy arrays: U (mt, 3) overwritten, y (mt, 3), f (n, 3), xn (n, 3);
    L, M, P: 3 entries; m: support half-width in standard deviations."""
    Lv = np.ascontiguousarray(np.broadcast_to(np.asarray(L, dtype=np.float64), (3,)))
    Mv = np.ascontiguousarray(np.broadcast_to(np.asarray(M, dtype=np.int32), (3,)))
    Pv = np.ascontiguousarray(np.broadcast_to(np.asarray(P, dtype=np.int32), (3,)))
    for a_ in (U, y, f, xn):
        _ptr(a_)
    check(lib().pb_fft_brinkman(U.ctypes.data_as(_dp), y.ctypes.data_as(_dp), int(y.shape[0]),
                                f.ctypes.data_as(_dp), xn.ctypes.data_as(_dp), int(xn.shape[0]),
                                Lv.ctypes.data_as(_dp), Mv.ctypes.data_as(_ip), Pv.ctypes.data_as(_ip), int(m), int(C_),
                                float(e), float(tol), float(d), float(alpha)))
    return U


def Brinkmanlet(y, x, f, alpha: float, eps: float = 0.0, U=None, stream=None):
    """Free-space velocities (m, 3) at y of forces f at x: the reference's
    Brinkmanlet (cuda/periodicBrinkman.h:119-141), regularized (eps > 0) or
    singular (eps = 0), summed directly on the GPU in FP64.  Host numpy or
    device torch buffers (all alike)."""
    m, n = int(y.shape[0]), int(x.shape[0])
    if U is None:
        if _is_torch(y):
            import torch

            U = torch.empty((m, 3), dtype=torch.float64, device=y.device)
        else:
            U = np.empty((m, 3))
    where = _where([y, x, f, U])
    s = None
    if stream is not None:
        s = stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)
    check(lib().pb_brinkmanlet(_ptr(U), _ptr(y), m, _ptr(x), _ptr(f), n, float(alpha), float(eps), where, s))
    return U


def brinkmanlet_matrix(dA, dx, dx0, alpha: float, eps: float = 0.0, stream=None):
    """dA (device, (3m, 3n) column-major) += the free-space Brinkmanlet tensors."""
    if not (_is_torch(dA) and dA.is_cuda):
        raise ValueError("brinkmanlet_matrix works on device tensors")
    m, n = int(dx.shape[0]), int(dx0.shape[0])
    if tuple(dA.shape) != (3 * m, 3 * n) or not dA.t().is_contiguous():
        raise ValueError("dA must be (3m, 3n) column-major")
    s = None
    if stream is not None:
        s = stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)
    check(lib().pb_brinkmanlet_matrix(dA.data_ptr(), _ptr(dx), m, _ptr(dx0), n, float(alpha), float(eps), s))
    return dA


def read_data(file_name: str, params: dict | None = None, delimiters: str = ": ") -> dict:
    """readData's map form (cuda/periodicBrinkman.cu:44-70): the file's
    "name<delimiters>value" lines into `params` (created if None; entries of
    names absent from the file keep their values, e.g. the defaults the
    reference's driver sets at cuda/periodicBrinkman.cu:78-87)."""
    params = {} if params is None else params
    cap = 64
    while True:
        keys = (C.c_char * 64 * cap)()
        vals = np.zeros(cap)
        n = lib().pb_read_param_file(str(file_name).encode(), delimiters.encode(), keys, vals.ctypes.data_as(_dp),
                                     cap)
        if n < 0:
            check(n)
        if n <= cap:
            break
        cap = n
    for k in range(n):
        params[bytes(keys[k]).split(b"\0", 1)[0].decode()] = float(vals[k])
    return params


def read_data_array(file_name: str, names, values=None, delimiters: str = ": "):
    """readData's array twin (cuda/periodicBrinkman.h:524-554): values[k] for names[k]."""
    names = list(names)
    vals = np.zeros(len(names)) if values is None else np.ascontiguousarray(values, dtype=np.float64)
    arr = (C.c_char_p * max(len(names), 1))(*[s.encode() for s in names])
    check(lib().pb_read_params(str(file_name).encode(), delimiters.encode(), arr, vals.ctypes.data_as(_dp),
                               len(names)))
    return vals


def shell_counts(L, M: int, N: int):
    """Per-axis (real, Fourier) shell counts used by periodicBrinkman
    (cuda/periodicBrinkman.h:457-487)."""
    L = [float(v) for v in np.broadcast_to(np.asarray(L, dtype=np.float64), (3,))]
    idL = [0, 1, 2]
    if L[idL[0]] > L[idL[1]]:
        idL[0], idL[1] = idL[1], idL[0]
    if L[idL[2]] <= L[idL[0]]:
        idL = [idL[2], idL[0], idL[1]]
    elif L[idL[2]] < L[idL[1]]:
        idL[1], idL[2] = idL[2], idL[1]
    Mx, Nx = [M] * 3, [N] * 3
    Mx[idL[2]] = int(np.ceil(M * L[idL[0]] / L[idL[2]]))
    Mx[idL[1]] = int(np.ceil(M * L[idL[0]] / L[idL[1]]))
    Nx[idL[0]] = int(np.ceil(N * L[idL[2]] / L[idL[0]]))
    Nx[idL[1]] = int(np.ceil(N * L[idL[2]] / L[idL[1]]))
    return Mx, Nx


def pair_kernel_tables64(alpha: float, d: float, eps: float, rc: float, r) -> tuple[np.ndarray, np.ndarray]:
    """H1(r), H2(r) of the FP64 path (FP64 far series beyond r_mid, closed forms
    below), evaluated on the host as the GPU does."""
    r = np.ascontiguousarray(r, dtype=np.float64)
    h1 = np.zeros_like(r)
    h2 = np.zeros_like(r)
    check(lib().pb_debug_pair_kernel64(alpha, d, eps, rc, r.size, r.ctypes.data_as(_dp), h1.ctypes.data_as(_dp),
                                       h2.ctypes.data_as(_dp)))
    return h1, h2


def pair_kernel_tables(alpha: float, d: float, eps: float, rc: float, r) -> tuple[np.ndarray, np.ndarray]:
    """H1(r), H2(r) of the FP32 polynomial tables, evaluated on the host as the
    GPU does (for testing the tables without a GPU)."""
    r = np.ascontiguousarray(r, dtype=np.float64)
    h1 = np.zeros_like(r)
    h2 = np.zeros_like(r)
    check(lib().pb_debug_pair_kernel(alpha, d, eps, rc, r.size, r.ctypes.data_as(_dp), h1.ctypes.data_as(_dp),
                                     h2.ctypes.data_as(_dp)))
    return h1, h2
