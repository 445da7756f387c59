"""GB300-native periodic regularized Brinkman evaluator (spectral Ewald).

The compute path is the CUDA library ``_lib/libpbrinkman.so`` (C ABI declared
in ``include/pbrinkman.h``), built by ``periodicbrinkman_gb300.build``.  This
module is the host-side mirror of the reference's entry points:

* ``periodicBrinkman(dA, dx, dx0, a, d, e, M, N, L, maxBlockSize=256)`` --
  the dense mobility matrix of cuda/periodicBrinkman.h:432-513 (device
  arrays, accumulates into dA);
* ``fftBrinkman(U, y, f, xn, L, M, P, m, C, e, tol, d, alpha=1)`` -- the
  k-space velocities of cuda/fftBrinkman.h:34-287 (host arrays, U overwritten);
* ``Brinkmanlet(y, x, f, alpha, eps)`` -- free-space velocities of the
  reference's Brinkmanlet (cuda/periodicBrinkman.h:119-141);

plus the full evaluator (real + k space + self), batched plans and the
continuous-batching server.  There is no CPU fallback: without the built
library or a CUDA device every compute call raises.
"""
from __future__ import annotations

from ._lib import (  # noqa: F401
    PB_DEVICE,
    PB_FLAGS_DEFAULT,
    PB_HOST,
    PB_KSPACE,
    PB_PREC_FP64,
    PB_PREC_MIXED,
    PB_REAL_SPACE,
    PB_ZERO_MODE,
    PbError,
    SolveParams,
    device_count,
    lib,
    lib_path,
)
from .api import (Brinkmanlet, Plan, Server, brinkmanlet_matrix, fftBrinkman, pair_kernel_tables,  # noqa: F401
                  pair_kernel_tables64, periodicBrinkman, read_data, read_data_array, shell_counts, solve,
                  tune_report)

__all__ = [
    "Brinkmanlet",
    "brinkmanlet_matrix",
    "PbError",
    "Plan",
    "Server",
    "SolveParams",
    "fftBrinkman",
    "periodicBrinkman",
    "solve",
    "shell_counts",
    "tune_report",
    "read_data",
    "read_data_array",
    "pair_kernel_tables",
    "pair_kernel_tables64",
    "device_count",
    "lib",
    "lib_path",
]
