"""GPU tests of forces-only executions (pb_plan_execute_forces): the plan
applied to new forces at the positions of its last full execution, as an
iterative solver's matrix-free mobility product.  Compared with full
executions (same plan, same positions) and with the FP64 oracle."""
import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import periodicbrinkman_gb300 as pb  # noqa: E402
from periodicbrinkman_gb300 import _lib  # noqa: E402
from periodicbrinkman_gb300.api import Plan, make_params  # noqa: E402

# atomics make the summation order vary between executions: relative to max |u|
TOL = {"mixed": 1e-6, "fp64": 1e-12}


def _inputs(n, m, seed):
    rng = np.random.default_rng(seed)
    x = rng.random((n, 3))
    fs = [rng.standard_normal((n, 3)) for _ in range(3)]
    y = rng.random((m, 3)) if m else None
    return x, fs, y


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
@pytest.mark.parametrize("m", [0, 700])
def test_forces_only_equals_full_execution(prec, m):
    x, (f1, f2, f3), y = _inputs(2000, m, 41)
    p = make_params(2000, 1.0, 10.0, 0.01, n_tgt=m, tol=1e-6 if prec == "mixed" else 1e-10, precision=prec)
    with Plan(p) as plan:
        full = [plan.execute(x, f, y=y).copy() for f in (f1, f2, f3)]
        plan.execute(x, f1, y=y)
        # eager, captured and replayed forces-only executions
        fo = [plan.execute_forces(f).copy() for f in (f2, f3, f2)]
    tol = TOL[prec]
    for got, ref in ((fo[0], full[1]), (fo[1], full[2]), (fo[2], full[1])):
        assert np.abs(got - ref).max() <= tol * np.abs(ref).max()


def test_forces_only_is_linear_and_accurate():
    x, (f1, f2, _), y = _inputs(3000, 500, 42)
    p = make_params(3000, 1.0, 5.0, 0.005, n_tgt=500, tol=1e-6, precision="mixed")
    with Plan(p) as plan:
        plan.execute(x, f1, y=y)
        u1 = plan.execute_forces(f1).copy()
        u2 = plan.execute_forces(f2).copy()
        u12 = plan.execute_forces(2.0 * f1 - 0.5 * f2).copy()
    assert np.abs(u12 - (2.0 * u1 - 0.5 * u2)).max() <= 2e-6 * np.abs(u12).max()
    sel = np.arange(0, 500, 25)
    ref = oracle.ewald_velocity(y[sel], x, f2, 1.0, 5.0, 0.005)
    assert oracle.rel_errors(u2[sel], ref)[0] < 1e-6


def test_forces_only_on_device_buffers_and_new_positions():
    x, (f1, f2, _), _ = _inputs(1500, 0, 43)
    x2 = np.random.default_rng(44).random((1500, 3))
    p = make_params(1500, 1.0, 10.0, 0.01, tol=1e-6, precision="mixed")
    with Plan(p) as plan:
        xd, f1d, f2d = (torch.from_numpy(a).cuda() for a in (x, f1, f2))
        for _ in range(3):  # through the captured graphs of both kinds
            plan.execute(xd, f1d)
            got = plan.execute_forces(f2d).cpu().numpy()
        ref = plan.execute(x, f2)
        assert np.abs(got - ref).max() <= 1e-6 * np.abs(ref).max()
        # new positions: the next forces-only execution uses them
        plan.execute(x2, f1)
        got2 = plan.execute_forces(f2)
        ref2 = plan.execute(x2, f2)
        assert np.abs(got2 - ref2).max() <= 1e-6 * np.abs(ref2).max()


def test_forces_only_needs_positions_and_finite_forces():
    x, (f1, _, _), _ = _inputs(500, 0, 45)
    p = make_params(500, 1.0, 10.0, 0.01, tol=1e-6, precision="mixed")
    with Plan(p) as plan:
        with pytest.raises(pb.PbError) as ei:
            plan.execute_forces(f1)
        assert ei.value.code == _lib.PB_ERR_INVALID
        ref = plan.execute(x, f1).copy()
        bad = f1.copy()
        bad[11, 0] = np.nan
        with pytest.raises(pb.PbError) as ei:
            plan.execute_forces(bad)
        assert ei.value.code == _lib.PB_ERR_INVALID
        again = plan.execute_forces(f1)
    assert np.abs(again - ref).max() <= 1e-6 * np.abs(ref).max()
