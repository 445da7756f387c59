"""ctypes binding of the C ABI in include/pbrinkman.h."""
from __future__ import annotations

import ctypes as C
import os
import re

_HERE = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(_HERE)
_LIB_PATH = os.path.join(_HERE, "_lib", "libpbrinkman.so")
_HEADER = os.path.join(_ROOT, "include", "pbrinkman.h")

PB_OK = 0
PB_ERR_INVALID = -1
PB_ERR_CUDA = -2
PB_ERR_NOMEM = -3
PB_ERR_UNSUPPORTED = -4
PB_ERR_BUDGET = -5
PB_ERR_BUSY = -6
PB_PREC_FP64 = 0
PB_PREC_MIXED = 1
PB_REAL_SPACE = 1
PB_KSPACE = 2
PB_ZERO_MODE = 4
PB_FLAGS_DEFAULT = PB_REAL_SPACE | PB_KSPACE
PB_HOST = 0
PB_DEVICE = 1
PB_HOST_PINNED = 2

_ERRNAMES = {
    PB_ERR_INVALID: "PB_ERR_INVALID",
    PB_ERR_CUDA: "PB_ERR_CUDA",
    PB_ERR_NOMEM: "PB_ERR_NOMEM",
    PB_ERR_UNSUPPORTED: "PB_ERR_UNSUPPORTED",
    PB_ERR_BUDGET: "PB_ERR_BUDGET",
    PB_ERR_BUSY: "PB_ERR_BUSY",
}


class PbError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_ERRNAMES.get(code, code)}: {msg}")
        self.code = code


class SolveParams(C.Structure):
    _fields_ = [
        ("n_src", C.c_int),
        ("n_tgt", C.c_int),
        ("L", C.c_double * 3),
        ("alpha", C.c_double),
        ("eps", C.c_double),
        ("tol", C.c_double),
        ("d", C.c_double),
        ("rc", C.c_double),
        ("M", C.c_int * 3),
        ("P", C.c_int),
        ("m_std", C.c_double),
        ("precision", C.c_int),
        ("flags", C.c_int),
    ]


class InstanceInfo(C.Structure):
    _fields_ = [
        ("d", C.c_double),
        ("rc", C.c_double),
        ("eta", C.c_double),
        ("m_std", C.c_double),
        ("M", C.c_int * 3),
        ("P", C.c_int),
        ("ncell", C.c_int * 3),
        ("npoly", C.c_int),
        ("pairs_est", C.c_longlong),
    ]


class SlotConfig(C.Structure):
    _fields_ = [
        ("M", C.c_int * 3),
        ("max_instances", C.c_int),
        ("max_src", C.c_int),
        ("max_tgt", C.c_int),
        ("max_cells", C.c_int),
        ("precision", C.c_int),
        ("npoly", C.c_int),
    ]


class TuneRow(C.Structure):
    _fields_ = [
        ("status", C.c_int),
        ("d", C.c_double),
        ("rc", C.c_double),
        ("M", C.c_int * 3),
        ("P", C.c_int),
        ("pairs_est", C.c_longlong),
        ("max_err", C.c_double),
        ("rms_err", C.c_double),
        ("ms", C.c_double),
    ]


class ServerConfig(C.Structure):
    _fields_ = [
        ("budget_bytes", C.c_longlong),
        ("precision", C.c_int),
        ("max_batch", C.c_int),
        ("slots_per_grid", C.c_int),
        ("n_grids", C.c_int),
        ("grids", C.c_int * 8),
        ("max_src", C.c_int),
        ("max_tgt", C.c_int),
        ("queue_capacity", C.c_int),
        ("linger_us", C.c_int),
        ("max_dynamic_per_grid", C.c_int),
        ("dynamic_idle_ms", C.c_int),
    ]


class ServerCounters(C.Structure):
    _fields_ = [
        ("submitted", C.c_longlong),
        ("completed", C.c_longlong),
        ("failed", C.c_longlong),
        ("rejected", C.c_longlong),
        ("batches", C.c_longlong),
        ("mean_batch", C.c_double),
        ("device_bytes", C.c_longlong),
        ("slots", C.c_int),
        ("kernels", C.c_longlong),
        ("scheduler_busy_s", C.c_double),
        ("peak_device_bytes", C.c_longlong),
        ("slots_created", C.c_longlong),
        ("slots_released", C.c_longlong),
        ("memory_waits", C.c_longlong),
    ]


_lib = None


def lib_path() -> str:
    return _LIB_PATH


def header_functions() -> list[str]:
    """Names of the functions declared in include/pbrinkman.h."""
    txt = open(_HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(pb_[a-z0-9_]+)\s*\(", txt)))


def lib():
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        raise RuntimeError(
            f"CUDA library not built: {_LIB_PATH} is missing (run periodicbrinkman_gb300/build.py or "
            "__graft_entry__.build())"
        )
    L = C.CDLL(_LIB_PATH)
    dp, ip, vp = C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_void_p
    L.pb_last_error.restype = C.c_char_p
    L.pb_version.restype = C.c_char_p
    L.pb_device_count.restype = C.c_int
    L.pb_periodic_brinkman.argtypes = [vp, vp, C.c_int, vp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int,
                                       C.c_int, dp, C.c_int]
    L.pb_periodic_brinkman_ex.argtypes = [vp, vp, C.c_int, vp, C.c_int, C.c_double, C.c_double, C.c_double, ip, ip,
                                          dp, C.c_int, vp]
    L.pb_fft_brinkman.argtypes = [dp, dp, C.c_int, dp, dp, C.c_int, dp, ip, ip, C.c_int, C.c_int, C.c_double,
                                  C.c_double, C.c_double, C.c_double]
    L.pb_fft_brinkman_static.argtypes = [vp, vp, C.c_int, vp, vp, C.c_int, dp, ip, ip, C.c_int, C.c_double,
                                         C.c_double, C.c_double, vp]
    L.pb_solve.argtypes = [C.POINTER(SolveParams), vp, vp, vp, vp, C.c_int, vp]
    L.pb_plan_create.argtypes = [C.POINTER(SolveParams), C.c_int, C.POINTER(vp)]
    L.pb_plan_execute.argtypes = [vp, vp, vp, vp, vp, C.c_int, vp]
    L.pb_plan_execute_forces.argtypes = [vp, vp, vp, C.c_int, vp]
    L.pb_plan_instance_info.argtypes = [vp, C.c_int, C.POINTER(InstanceInfo)]
    L.pb_resolve.argtypes = [C.POINTER(SolveParams), C.POINTER(InstanceInfo)]
    L.pb_plan_device_bytes.restype = C.c_longlong
    L.pb_plan_device_bytes.argtypes = [vp]
    L.pb_plan_kernel_count.argtypes = [vp]
    L.pb_plan_estimate_bytes.restype = C.c_longlong
    L.pb_plan_estimate_bytes.argtypes = [C.POINTER(SolveParams), C.c_int]
    L.pb_plan_set_timing.argtypes = [vp, C.c_int]
    L.pb_plan_status.argtypes = [vp]
    L.pb_plan_set_item_capacity.argtypes = [vp, C.c_int]
    L.pb_plan_stage_ms.argtypes = [vp, dp]
    L.pb_plan_destroy.argtypes = [vp]
    L.pb_debug_pair_kernel.argtypes = [C.c_double] * 4 + [C.c_int, dp, dp, dp]
    L.pb_debug_pair_kernel64.argtypes = [C.c_double] * 4 + [C.c_int, dp, dp, dp]
    L.pb_debug_fft_green.argtypes = [C.POINTER(SolveParams), vp, vp]
    L.pb_read_params.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(C.c_char_p), dp, C.c_int]
    L.pb_read_param_file.argtypes = [C.c_char_p, C.c_char_p, C.c_void_p, dp, C.c_int]
    L.pb_tune_report.argtypes = [C.POINTER(SolveParams), vp, vp, vp, C.c_int, dp, C.c_int, C.c_double,
                                 C.POINTER(TuneRow)]
    L.pb_brinkmanlet.argtypes = [vp, vp, C.c_int, vp, vp, C.c_int, C.c_double, C.c_double, C.c_int, vp]
    L.pb_brinkmanlet_matrix.argtypes = [vp, vp, C.c_int, vp, C.c_int, C.c_double, C.c_double, vp]
    L.pb_plan_create_slot.argtypes = [C.POINTER(SlotConfig), C.POINTER(vp)]
    L.pb_slot_estimate_bytes.restype = C.c_longlong
    L.pb_slot_estimate_bytes.argtypes = [C.POINTER(SlotConfig)]
    L.pb_plan_bind.argtypes = [vp, C.POINTER(SolveParams), C.c_int]
    L.pb_server_create.argtypes = [C.POINTER(ServerConfig), C.POINTER(vp)]
    L.pb_server_submit.argtypes = [vp, C.POINTER(SolveParams), vp, vp, vp, vp, C.POINTER(C.c_longlong)]
    L.pb_server_poll.argtypes = [vp, C.c_longlong, ip, ip, dp]
    L.pb_server_wait.argtypes = [vp, C.c_longlong, C.c_double, ip, dp]
    L.pb_server_release.argtypes = [vp, C.c_longlong]
    L.pb_server_drain.argtypes = [vp, C.c_double]
    L.pb_server_stats.argtypes = [vp, C.POINTER(ServerCounters)]
    L.pb_server_destroy.argtypes = [vp]
    _lib = L
    return L


def check(rc: int) -> None:
    if rc != PB_OK:
        raise PbError(rc, lib().pb_last_error().decode())


def device_count() -> int:
    return int(lib().pb_device_count())
