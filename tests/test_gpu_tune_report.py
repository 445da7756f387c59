"""pb_tune_report: measured error against the splitting width, the study of
the reference's driver (cuda/periodicBrinkman.cu:139-203: the Ewald total is
the same for every splitting width d) run on the GPU against an FP64
reference solution of the same instance."""
import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import periodicbrinkman_gb300 as pb  # noqa: E402
from periodicbrinkman_gb300.api import make_params, resolve  # noqa: E402


@pytest.mark.parametrize("prec,tol", [("mixed", 1e-6), ("fp64", 1e-10)])
def test_splitting_independence_report(prec, tol):
    rng = np.random.default_rng(81)
    n, alpha, eps = 3000, 10.0, 0.01
    x, f = rng.random((n, 3)), rng.standard_normal((n, 3))
    ds = [0.0, 0.03, 0.045, 0.07]
    rows = pb.tune_report(x, f, 1.0, alpha, eps, d_values=ds, tol=tol, precision=prec)
    assert len(rows) == len(ds)
    auto = resolve(make_params(n, 1.0, alpha, eps, tol=tol, precision=prec))
    assert rows[0]["d"] == pytest.approx(auto["d"]) and rows[0]["M"] == auto["M"]
    for d, r in zip(ds, rows):
        assert r["status"] == 0, r
        if d > 0:
            assert r["d"] == pytest.approx(d)
        assert 0 <= r["max_err"] < tol and 0 <= r["rms_err"] <= r["max_err"], (d, r)
        assert r["ms"] > 0 and r["pairs_est"] > 0
    # the reference solution itself against the oracle
    sel = np.arange(0, n, 100)
    u = pb.solve(x, f, 1.0, alpha, eps, tol=1e-12, precision="fp64")
    assert oracle.rel_errors(u[sel], oracle.ewald_velocity(x[sel], x, f, 1.0, alpha, eps))[0] < 1e-11


def test_tune_report_flags_a_choice_that_misses_the_tolerance():
    rng = np.random.default_rng(82)
    n = 2000
    x, f, y = rng.random((n, 3)), rng.standard_normal((n, 3)), rng.random((500, 3))
    # fully autotuned: within the tolerance
    ok = pb.tune_report(x, f, 1.0, 5.0, 0.005, y=y, d_values=[0.0], tol=1e-6)
    assert ok[0]["status"] == 0 and ok[0]["max_err"] < 1e-6, ok
    # a support of 8 points fixed on a fixed 32^3 grid cannot reach 1e-6 for any
    # splitting width (window truncation and aliasing): the report shows it
    rows = pb.tune_report(x, f, 1.0, 5.0, 0.005, y=y, d_values=[0.0, 0.02], tol=1e-6, M=32, P=8)
    for r in rows:
        assert r["status"] != 0 or r["max_err"] > 1e-6, r
    assert rows[0]["status"] == 0 and rows[0]["M"] == [32, 32, 32] and rows[0]["P"] == 8
