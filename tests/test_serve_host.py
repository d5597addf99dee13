"""Host-side tests of the request loop (ecs_serve.h) that need no GPU:
admission charges, refusals at submit, argument checks, and the failure path
(a request whose context cannot come up is returned with its error, the
server stays usable and its slot is released)."""
import numpy as np
import pytest

import ecsprt_gb300 as E
from ecsprt_gb300 import workloads as W

from conftest import have_gpu


def params(n):
    return E.params_from_options(W.solver_options(n))


def test_request_bytes(built):
    b = [E.serve_request_bytes(params(n)) for n in W.SOLVE_SIZES]
    assert all(x < y for x, y in zip(b, b[1:]))
    n = 128 ** 3
    # mixed solve slot: FGMRES(30) FP32 bases + FP64 fields + multigrid, a few hundred bytes a cell
    assert 300 * n < b[-1] < 600 * n
    assert E.serve_request_bytes(params(64), E.ECS_PREC_FP64) > E.serve_request_bytes(params(64))
    p = E.params_from_options(W.sim_options(32, 16, 1.0, 0.02))
    ions = 32 ** 3 * 16
    sim = E.serve_request_bytes(p, E.ECS_PREC_MIXED, E.ECS_SERVE_SIM, ions)
    solve = E.serve_request_bytes(p, E.ECS_PREC_MIXED, E.ECS_SERVE_SOLVE, ions)
    # two 32-byte records, a sort key and a permutation entry an ion, plus five
    # staging buffers (two in, three out) of a position and a velocity region
    # of 3 doubles an ion and 64 doubles of alignment room each
    chunk = max(ions // 8, 1 << 16)
    assert sim - solve == 72 * ions + 5 * 2 * (3 * chunk + 64) * 8
    assert E.serve_request_bytes(params(16)) > 8 << 20  # fixed allowance: rounding, graphs


def test_submit_refusals(built):
    with E.Server(hbm_budget_bytes=E.serve_request_bytes(params(32)), max_inflight=2) as srv:
        big = np.zeros((48, 48, 48))
        with pytest.raises(E.EcsError) as ei:
            srv.submit_solve(params(48), big, np.empty_like(big))
        assert ei.value.code == E._lib.ECS_ERR_NOMEM
        d = np.zeros((32, 32, 32))
        with pytest.raises(ValueError):
            srv.submit_solve(params(32), d.astype(np.float32), np.empty_like(d))
        with pytest.raises(ValueError):
            srv.submit_solve(params(32), d, np.empty((16, 16, 16)))
        with pytest.raises(E.EcsError) as ei:
            srv.submit_solve(params(32), d, np.empty_like(d), rtol=0.0)
        assert ei.value.code == E._lib.ECS_ERR_INVALID
        pos = np.zeros((10, 3))
        with pytest.raises(E.EcsError) as ei:
            srv.submit_sim(params(32), pos, pos.copy(), 0, 0.1)
        assert ei.value.code == E._lib.ECS_ERR_INVALID
        assert srv.pending == 0


def test_server_config_checks(built):
    for kw in ({"hbm_budget_bytes": 0}, {"hbm_budget_bytes": 1 << 30, "max_inflight": 0},
               {"hbm_budget_bytes": 1 << 30, "precision": 7}):
        with pytest.raises(E.EcsError):
            E.Server(**kw)


@pytest.mark.skipif(have_gpu(), reason="checks the no-device failure path")
def test_failed_requests_come_back_in_order(built):
    """Without a device every context creation fails: each request returns
    ECS_ERR_CUDA with its message, in submission order (one worker), and the
    slots it was charged are released."""
    budget = 3 * E.serve_request_bytes(params(24))
    with E.Server(hbm_budget_bytes=budget, max_inflight=1) as srv:
        d = np.zeros((24, 24, 24))
        ids = [srv.submit_solve(params(24), d, np.empty_like(d)) for _ in range(5)]
        res = srv.wait_all(30)
        st = srv.stats()
    assert [r["id"] for r in res] == ids
    assert all(r["status"] == E._lib.ECS_ERR_CUDA and r["message"] for r in res)
    assert st["failed"] == 5 and st["completed"] == 0 and st["solves"] == 0
    assert st["device_bytes"] == 0 and st["slots"] == 0
    assert st["peak_device_bytes"] <= budget


def test_workload_generators():
    t, n = W.solve_requests(2000, 200.0, seed=1)
    assert t[0] == 0.0 and np.all(np.diff(t) >= 0)
    assert abs(t[-1] / 1999 - 1 / 200.0) < 0.1 / 200.0  # mean gap 5 ms
    assert set(np.unique(n)) == set(W.SOLVE_SIZES)
    d = W.solve_density(16, np.random.default_rng(2))
    assert d.shape == (16, 16, 16) and d.min() > 0
    assert abs(np.log(d).mean()) < 0.05
    inst = W.sim_instances(48, seed=3)
    assert len(inst) == 48
    assert all(n in W.SIM_SIZES and 0.2 <= v <= 1.5 and 0.005 <= nu <= 0.1 for n, v, nu in inst)
    m = W.fourier_modes((8, 8, 8), 3, 0.05, np.random.default_rng(4))
    assert np.abs(m).max() <= 0.15 + 1e-12 and abs(m.mean()) < 1e-12
