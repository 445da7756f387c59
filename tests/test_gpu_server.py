"""GPU tests of capacity plans (slots), instance binding and the
continuous-batching server: every result is the same alone and in the mix
within the stated tolerance, and accurate against the FP64 oracle."""
import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import periodicbrinkman_gb300 as pb  # noqa: E402
from periodicbrinkman_gb300 import _lib  # noqa: E402
from periodicbrinkman_gb300.api import Server, bind, make_params, make_slot, resolve, slot_estimate_bytes  # noqa: E402

MIX_TOL = 1e-6  # alone vs in the mix, relative to max |u|


def _req(rng, n, L, sep):
    x = rng.random((n, 3)) * L
    f = rng.standard_normal((n, 3))
    y = rng.random((n // 2, 3)) * L if sep else None
    a = float(np.exp(rng.uniform(0, np.log(50))))
    e = float(np.exp(rng.uniform(np.log(1e-3), np.log(1e-2)))) * L
    return x, f, y, a, e


def _cuda(a):
    return None if a is None else torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_slot_binding_matches_fixed_plans():
    rng = np.random.default_rng(31)
    slot = make_slot(32, max_instances=6, max_src=6000, max_tgt=6000, max_cells=1 << 16)
    for rnd in range(3):
        reqs = [_req(rng, int(rng.integers(200, 900)), 1.0, sep=(k % 2 == 1)) for k in range(int(rng.integers(1, 6)))]
        params = [make_params(x.shape[0], 1.0, a, e, n_tgt=0 if y is None else y.shape[0], tol=1e-6, M=32)
                  for x, f, y, a, e in reqs]
        bind(slot, params)
        X = np.concatenate([r[0] for r in reqs])
        F = np.concatenate([r[1] for r in reqs])
        ys = [r[2] for r in reqs if r[2] is not None]
        Y = np.concatenate(ys) if ys else None
        U = slot.execute(_cuda(X), _cuda(F), _cuda(Y)).cpu().numpy()
        off = 0
        for (x, f, y, a, e) in reqs:
            u1 = pb.solve(_cuda(x), _cuda(f), 1.0, a, e, y=_cuda(y), tol=1e-6, M=32).cpu().numpy()
            m = u1.shape[0]
            assert np.abs(U[off:off + m] - u1).max() <= MIX_TOL * np.abs(u1).max(), (rnd, a, e)
            off += m
    slot.close()


def test_slot_capacity_is_enforced():
    slot = make_slot(16, max_instances=2, max_src=1000, max_tgt=1000, max_cells=4096)
    ps = [make_params(800, 1.0, 5.0, 0.01, tol=1e-6, M=16), make_params(800, 1.0, 5.0, 0.01, tol=1e-6, M=16)]
    with pytest.raises(pb.PbError) as ei:
        bind(slot, ps)
    assert ei.value.code == _lib.PB_ERR_BUDGET
    with pytest.raises(pb.PbError):
        bind(slot, [make_params(100, 1.0, 5.0, 0.01, M=32)])  # wrong grid for the slot
    slot.close()


def test_server_mix_equals_alone_and_oracle():
    rng = np.random.default_rng(32)
    # a 50 ms batching window: the burst of 24 requests is batched whatever the GPU speed
    with Server(precision="mixed", budget_bytes=8 << 30, max_batch=8, slots_per_grid=2, grids=(16, 32, 64),
                max_src=20000, max_tgt=20000, linger_us=50000) as srv:
        reqs, tickets = [], []
        for k in range(24):
            n = int(np.exp(rng.uniform(np.log(300), np.log(3000))))
            r = _req(rng, n, 1.0, sep=(k % 3 == 0))
            reqs.append(r)
            x, f, y, a, e = r
            tickets.append(srv.submit(x, f, 1.0, a, e, y=y, tol=1e-6))
        outs = [srv.result(t) for t in tickets]
        st = srv.stats()
        assert st["completed"] == 24 and st["failed"] == 0
        assert st["batches"] < 24  # requests were batched
    for k, ((x, f, y, a, e), (U, lat)) in enumerate(zip(reqs, outs)):
        assert lat > 0
        ref = oracle.ewald_velocity(x if y is None else y, x, f, 1.0, a, e)
        assert oracle.rel_errors(U, ref)[0] < 1e-6, k
        alone = pb.solve(_cuda(x), _cuda(f), 1.0, a, e, y=_cuda(y), tol=1e-6).cpu().numpy()
        assert np.abs(U - alone).max() <= 2 * MIX_TOL * np.abs(alone).max(), k


def test_server_rejects_and_validates():
    with Server(precision="mixed", budget_bytes=64 << 20, max_batch=4, slots_per_grid=1, grids=(16, 32),
                max_src=2000) as srv:
        rng = np.random.default_rng(33)
        x = rng.random((400_000, 3))
        with pytest.raises(pb.PbError) as ei:
            srv.submit(x, x.copy(), 1.0, 10.0, 0.01, tol=1e-6, M=32)  # a slot of its own exceeds the budget
        assert ei.value.code == _lib.PB_ERR_BUDGET
        assert srv.stats()["peak_device_bytes"] <= 64 << 20
        with pytest.raises(pb.PbError):
            srv.submit(x[:10], x[:10].copy(), 1.0, -1.0, 0.01)
        t = srv.submit(x[:100], x[:100].copy(), 1.0, 10.0, 0.01, tol=1e-6)
        U, _ = srv.result(t)
        assert np.isfinite(U).all()
        assert srv.stats()["rejected"] >= 1


def test_server_non_finite_request_fails_alone():
    """A request with a NaN position or force is found on the device and fails
    with PB_ERR_INVALID; the requests batched with it are unaffected."""
    with Server(precision="mixed", budget_bytes=2 << 30, max_batch=4, slots_per_grid=1, grids=(16, 32),
                max_src=2000, linger_us=50000) as srv:
        rng = np.random.default_rng(34)
        xs = [rng.random((300, 3)) for _ in range(3)]
        fs = [rng.standard_normal((300, 3)) for _ in range(3)]
        fs[1][7, 2] = np.nan
        tickets = [srv.submit(xs[k], fs[k], 1.0, 10.0, 0.01, tol=1e-6) for k in range(3)]
        for k in (0, 2):
            U, _ = srv.result(tickets[k])
            alone = pb.solve(_cuda(xs[k]), _cuda(fs[k]), 1.0, 10.0, 0.01, tol=1e-6).cpu().numpy()
            assert np.abs(U - alone).max() <= 2 * MIX_TOL * np.abs(alone).max(), k
        with pytest.raises(pb.PbError) as ei:
            srv.result(tickets[1])
        assert ei.value.code == _lib.PB_ERR_INVALID
        assert srv.stats()["failed"] >= 1


def test_server_admits_by_memory_budget():
    """Two requests larger than the resident slots, on different grids, with a
    budget that holds the resident slots and ONE slot for such a request: the
    first gets a dynamic slot at once, the second waits until that slot's
    memory is released, and both complete; the slots never hold more device
    memory than the budget."""
    # one instance per slot execution: the resident slots' size does not depend on the budget
    n, grids, res = 30000, (32, 64), dict(max_batch=1, slots_per_grid=1, max_src=2000)
    with Server(precision="mixed", budget_bytes=64 << 30, grids=grids, max_dynamic_per_grid=-1, **res) as probe:
        resident = probe.stats()["device_bytes"]
    need = 0
    for g in grids:
        info = resolve(make_params(n, 1.0, 10.0, 0.01, n_tgt=n // 2, tol=1e-6, M=g))
        cells = int(np.prod(info["ncell"]))
        need = max(need, slot_estimate_bytes(g, 1, n, n // 2, max(cells, (g // 2) ** 3)))
    budget = resident + need + need // 2
    rng = np.random.default_rng(35)
    reqs = [(rng.random((n, 3)), rng.standard_normal((n, 3)), rng.random((n // 2, 3)), g) for g in grids]
    with Server(precision="mixed", budget_bytes=budget, grids=grids, dynamic_idle_ms=60000, **res) as srv:
        assert srv.stats()["device_bytes"] == resident
        tickets = [srv.submit(x, f, 1.0, 10.0, 0.01, y=y, tol=1e-6, M=g) for x, f, y, g in reqs]
        outs = [srv.result(t, timeout=600)[0] for t in tickets]
        st = srv.stats()
    assert st["completed"] == 2 and st["failed"] == 0 and st["rejected"] == 0
    assert st["slots_created"] >= 2 and st["slots_released"] >= 1 and st["memory_waits"] >= 1, st
    assert st["peak_device_bytes"] <= budget, (st["peak_device_bytes"], budget)
    for (x, f, y, g), U in zip(reqs, outs):
        alone = pb.solve(_cuda(x), _cuda(f), 1.0, 10.0, 0.01, y=_cuda(y), tol=1e-6, M=g).cpu().numpy()
        assert np.abs(U - alone).max() <= MIX_TOL * np.abs(alone).max(), g
