"""GPU tests of the stand-alone solve and of the request loop (ecs_serve.h).

Tolerances:
  moments from a density       bit-exact (fluxes = 0 + flux_scale * density,
                               src/file-io.c:51-59)
  RHS                          <= 1e-14 relative against the oracle
  potential                    relres <= rtol, re-measured with the oracle's
                               FP64 operator (<= 2 rtol); FP64 path solved to
                               1e-11: phi relative L2 <= 1e-8 against the
                               oracle's 1e-13 GMRES solve
  graph vs step-by-step path   bit-exact (same kernels, same order)
  served vs alone              bit-exact: potentials of solve requests, and
                               final ions and potential of simulations (ions
                               compared as sets: the cell sort places ions of
                               one cell in arrival order, and nothing computed
                               depends on that order)
"""
import numpy as np
import pytest

import ecsprt_gb300 as E
from ecsprt_gb300 import workloads as W
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def solve_params(n):
    return E.params_from_options(W.solver_options(n))


def moments_of(density, fs):
    return np.stack([density] + [0.0 + f * density for f in fs], axis=-1)


@pytest.mark.parametrize("prec", [E.ECS_PREC_FP64, E.ECS_PREC_MIXED])
def test_solve_density_matches_oracle(built, prec):
    n = 24
    p = solve_params(n)
    rng = np.random.default_rng(11)
    dens = W.solve_density(n, rng)
    fs = (1.0, 0.5, -0.25)
    O = orc.Oracle(p)
    mom = moments_of(dens, fs)
    b_o = O.rhs(mom)
    phi_o, _, rel_o = O.solve(dens, b_o, rtol=1e-13)
    assert rel_o <= 1e-13
    rtol = 1e-11 if prec == E.ECS_PREC_FP64 else 1e-8
    with E.Context(p, prec) as ctx:
        phi, st = ctx.solve_density(dens, fs, rtol=rtol, max_it=400)
        assert np.array_equal(ctx.moments, mom)
        b = ctx.rhs
    assert np.abs(b - b_o).max() <= 1e-14 * np.abs(b_o).max()
    assert st.relres <= rtol
    r = b_o - O.lhs_apply(dens, phi)
    assert np.linalg.norm(r) / np.linalg.norm(b_o) <= 2 * rtol
    if prec == E.ECS_PREC_FP64:
        assert np.linalg.norm(phi - phi_o) / np.linalg.norm(phi_o) <= 1e-8


@pytest.mark.parametrize("prec", [E.ECS_PREC_FP64, E.ECS_PREC_MIXED])
def test_solve_density_graph_matches_stepwise(built, prec):
    """One request graph (copy in, fluxes, RHS, set-up, solve, copy out)
    gives the bits of the separate calls; repeated requests on one context
    too, and page-locked and pageable buffers alike."""
    n = 32
    p = solve_params(n)
    dens = W.solve_density(n, np.random.default_rng(12))
    with E.Context(p, prec) as ctx:
        ctx.moments = moments_of(dens, (1.0, 1.0, 1.0))
        st0 = ctx.compute_potential(rtol=1e-8, max_it=400)
        phi0 = ctx.phi
    with E.Context(p, prec) as ctx:
        phi1, st1 = ctx.solve_density(dens, rtol=1e-8, max_it=400)
        hd = E.pinned_empty(dens.shape)
        hd[:] = dens
        hphi = E.pinned_empty(dens.shape)
        _, st2 = ctx.solve_density(hd, rtol=1e-8, max_it=400, phi_out=hphi)
        phi2 = hphi.copy()
        phi3, _ = ctx.solve_density(dens, rtol=1e-8, max_it=400)
    assert (st0.iterations, st0.refinements) == (st1.iterations, st1.refinements) == (st2.iterations, st2.refinements)
    assert np.array_equal(phi0, phi1)
    assert np.array_equal(phi1, phi2)
    assert np.array_equal(phi1, phi3)


def _alone(params_list, dens_list, prec=E.ECS_PREC_MIXED):
    out = []
    for p, d in zip(params_list, dens_list):
        with E.Context(p, prec) as ctx:
            phi, st = ctx.solve_density(d, rtol=1e-8, max_it=400)
            out.append((phi.copy(), st.iterations))
    return out


def test_serve_solves_alone_vs_mix(built):
    """Uneven grids submitted together (several on the GPU at once, slots
    reused) give the same bits as each request alone."""
    rng = np.random.default_rng(13)
    sizes = [16, 24, 32, 48, 16, 32, 24, 48, 32, 16, 24, 32]
    params = {n: solve_params(n) for n in set(sizes)}
    dens = [W.solve_density(n, rng) for n in sizes]
    ref = _alone([params[n] for n in sizes], dens)
    with E.Server(hbm_budget_bytes=4 << 30, max_inflight=4) as srv:
        outs = [np.empty_like(d) for d in dens]
        ids = [srv.submit_solve(params[n], d, o) for n, d, o in zip(sizes, dens, outs)]
        res = {r["id"]: r for r in srv.wait_all(300)}
        st = srv.stats()
    assert all(res[i]["status"] == 0 for i in ids), [res[i]["message"] for i in ids]
    for q, i in enumerate(ids):
        assert np.array_equal(outs[q], ref[q][0]), f"request {q} (n={sizes[q]}) differs"
        assert res[i]["iterations"] == ref[q][1]
        assert res[i]["relres"] <= 1e-8
    assert st["solves"] == len(sizes) and st["failed"] == 0
    assert st["slot_hits"] > 0
    assert st["peak_inflight"] >= 2
    assert 0 < st["solve_p50"] <= st["solve_p99"]


def test_serve_budget_admission(built):
    """A budget one byte short of a 32^3 slot beside a 24^3 slot: the two
    sizes alternate, so every change of size waits for the other slot to go
    idle and evicts it (whatever the timing of the solves), the budget is
    never exceeded, and a request larger than the budget is refused at
    submit."""
    p32, p24, p64 = solve_params(32), solve_params(24), solve_params(64)
    b32 = E.serve_request_bytes(p32)
    b24 = E.serve_request_bytes(p24)
    budget = b32 + b24 - 1
    rng = np.random.default_rng(14)
    sizes = [32, 24, 32, 24, 32, 32, 24, 32]
    dens = [W.solve_density(n, rng) for n in sizes]
    ref = _alone([p32 if n == 32 else p24 for n in sizes], dens)
    with E.Server(hbm_budget_bytes=budget, max_inflight=3) as srv:
        with pytest.raises(E.EcsError) as ei:
            srv.submit_solve(p64, W.solve_density(64, rng), np.empty((64, 64, 64)))
        assert ei.value.code == E._lib.ECS_ERR_NOMEM
        outs = [np.empty_like(d) for d in dens]
        ids = [srv.submit_solve(p32 if n == 32 else p24, d, o) for n, d, o in zip(sizes, dens, outs)]
        res = {r["id"]: r for r in srv.wait_all(300)}
        st = srv.stats()
    assert all(res[i]["status"] == 0 for i in ids)
    for q in range(len(sizes)):
        assert np.array_equal(outs[q], ref[q][0])
    assert st["peak_device_bytes"] <= budget
    assert b24 < b32
    assert st["evictions"] > 0


def _rows_sorted(pos, vel):
    a = np.concatenate([pos, vel], axis=1)
    return a[np.lexsort(a.T[::-1])]


def _sim_inputs(n, ppc, drift, nu, seed):
    p = E.params_from_options(W.sim_options(n, ppc, drift, nu))
    pos, vel = W.uniform_ions(n, ppc, drift, np.random.default_rng(seed))
    return p, pos, vel


def test_serve_sims_match_direct_steps(built):
    """Simulation instances served together with solve requests end in the
    same state (ions and potential, bit for bit) as stepping a context
    directly; per-step wall times are reported."""
    specs = [(16, 8, 0.5, 0.05, 1), (24, 4, 1.2, 0.01, 2), (16, 8, 0.9, 0.1, 3)]
    nsteps = 6
    ref = []
    for n, ppc, drift, nu, seed in specs:
        p, pos, vel = _sim_inputs(n, ppc, drift, nu, seed)
        with E.Context(p, E.ECS_PREC_MIXED, np_capacity=pos.shape[0]) as ctx:
            ctx.set_seed(100 + seed)
            ctx.upload_particles(pos, vel)
            for _ in range(nsteps):
                ctx.step(0.1, 1e-8, 400)
            ref.append(ctx.download_particles() + (ctx.phi,))
    rng = np.random.default_rng(15)
    with E.Server(hbm_budget_bytes=4 << 30, max_inflight=3) as srv:
        sims = []
        for n, ppc, drift, nu, seed in specs:
            p, pos, vel = _sim_inputs(n, ppc, drift, nu, seed)
            o = dict(step_seconds=np.zeros(nsteps), phi_out=np.empty((n, n, n)),
                     pos_out=np.empty_like(pos), vel_out=np.empty_like(vel))
            sims.append((srv.submit_sim(p, pos, vel, nsteps, 0.1, seed=100 + seed, **o), o))
        for n in (16, 24, 32):  # solves arriving while the instances run
            d = W.solve_density(n, rng)
            srv.submit_solve(solve_params(n), d, np.empty_like(d))
        res = {r["id"]: r for r in srv.wait_all(300)}
        st = srv.stats()
    assert all(r["status"] == 0 for r in res.values()), [r["message"] for r in res.values()]
    for (rid, o), (pos_r, vel_r, phi_r) in zip(sims, ref):
        assert res[rid]["steps"] == nsteps
        assert np.array_equal(_rows_sorted(o["pos_out"], o["vel_out"]), _rows_sorted(pos_r, vel_r))
        assert np.array_equal(o["phi_out"], phi_r)
        assert (o["step_seconds"] > 0).all()
    assert st["steps"] == nsteps * len(specs)
    assert st["solves"] == 3


def test_serve_request_bytes_cover_allocation(built):
    """The admission charge of a slot is at least what its context holds on
    the device once a request has run on it."""
    import torch

    torch.cuda.init()
    for n, prec in ((64, E.ECS_PREC_MIXED), (48, E.ECS_PREC_FP64)):
        p = solve_params(n)
        charge = E.serve_request_bytes(p, prec)
        with E.Context(solve_params(16), prec) as warm:  # kernels loaded before measuring
            warm.solve_density(W.solve_density(16, np.random.default_rng(0)), rtol=1e-8, max_it=400)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        ctx = E.Context(p, prec)
        ctx.solve_density(W.solve_density(n, np.random.default_rng(16)), rtol=1e-8, max_it=400)
        torch.cuda.synchronize()
        held = free0 - torch.cuda.mem_get_info()[0]
        ctx.close()
        print(f"n={n} prec={prec}: charge {charge / 2**20:.1f} MiB, held {held / 2**20:.1f} MiB")
        assert held <= charge, (n, prec, held, charge)
        assert charge <= 1.3 * held + (16 << 20), (n, prec, held, charge)
