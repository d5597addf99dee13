"""GPU parity of the 2-D path (-ndim 2) against the reference's golden
vectors (tests/golden/twod.npz) and the oracle.

Tolerances (as the 3-D path):
  FP64  push, move            bit-exact
        deposit               bit-exact against the oracle's fixed-point
                              deposit; <= 1e-13 relative (density) and
                              64 flux quanta against the reference's FP64 sums
        RHS                   <= 1e-14 relative
        operator apply        <= 1e-13 relative against the reference's matrix
        solve                 relres <= rtol, re-measured with the reference's
                              matrix
  mixed push velocities       <= 2e-6 x max|v|; positions <= 2e-6 cell widths;
        density               <= 1e-6 relative
  larger runs                 ion count conserved, relres <= 1e-8
"""
import json

import numpy as np
import pytest

import ecsprt_gb300 as E
from conftest import GOLDEN
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g2():
    d = dict(np.load(GOLDEN / "twod.npz"))
    d["opts"] = str(d["opts"])
    d["params"] = json.loads(str(d["params"]))
    return d


def ctx_for(g, prec, n=None):
    p = E.params_from_options(g["opts"])
    ctx = E.Context(p, prec, np_capacity=n if n is not None else g["pos0"].shape[0])
    ctx.set_sort_every(0)
    return ctx


def fix_shifts(p, prec):
    import ctypes
    from ecsprt_gb300 import _lib
    sn, sf = ctypes.c_int32(), ctypes.c_int32()
    assert _lib.gpu().ecs_fix_shifts(ctypes.byref(p), prec, ctypes.byref(sn), ctypes.byref(sf)) == 0
    return sn.value, sf.value


def test_fp64_push_move_bit_exact(built, g2):
    dt = float(g2["dt"])
    with ctx_for(g2, E.ECS_PREC_FP64) as ctx:
        ctx.upload_particles(g2["pos0"], g2["vel0"])
        ctx.phi = g2["phi"]
        ctx.push(dt)
        _, vel = ctx.download_particles()
        assert np.array_equal(vel, g2["vel_push"])
        ctx.upload_particles(g2["pos0"], g2["vel_push"])
        ctx.update_positions(dt)
        pos, vel = ctx.download_particles()
    assert np.array_equal(pos, g2["pos_move"])
    assert np.array_equal(vel, g2["vel_move"])


def test_fp64_deposit(built, g2):
    p = E.params_from_options(g2["opts"])
    with ctx_for(g2, E.ECS_PREC_FP64) as ctx:
        ctx.upload_particles(g2["pos_move"], g2["vel_move"])
        ctx.collect()
        m = ctx.moments
    sn, sf = fix_shifts(p, E.ECS_PREC_FP64)
    m_fix, _ = orc.Oracle(g2["params"]).collect_fixed(g2["pos_move"], g2["vel_move"], sn, sf)
    assert np.array_equal(m, m_fix)
    ref = g2["moments"]
    assert np.abs(m[..., 0] - ref[..., 0]).max() <= 1e-13 * np.abs(ref[..., 0]).max()
    assert np.abs(m[..., 1:] - ref[..., 1:]).max() <= 64 * 2.0 ** -sf
    assert np.all(m[..., 3] == 0)


@pytest.mark.parametrize("prec", [E.ECS_PREC_FP64, E.ECS_PREC_MIXED])
def test_rhs_operator_solve(built, g2, prec):
    A = g2["lhs"]
    with ctx_for(g2, prec) as ctx:
        ctx.moments = g2["moments"]
        ctx.compute_rhs()
        b = ctx.rhs
        ctx.compute_lhs()
        x = np.random.default_rng(4).standard_normal(b.shape)
        y = ctx.lhs_apply(x)
        rtol = 1e-11 if prec == E.ECS_PREC_FP64 else 1e-8
        st = ctx.solve(rtol=rtol, max_it=200)
        phi = ctx.phi
    assert np.abs(b - g2["rhs"]).max() <= 1e-14 * np.abs(g2["rhs"]).max()
    y_ref = (A @ x.ravel()).reshape(x.shape)
    assert np.abs(y - y_ref).max() <= 1e-13 * np.abs(y_ref).max()
    r = g2["rhs"].ravel() - A @ phi.ravel()
    assert st.relres <= rtol
    assert np.linalg.norm(r) / np.linalg.norm(g2["rhs"]) <= 2 * rtol


def test_laplacian_sinusoidal_2d(built, g2):
    p = E.params_from_options(str(g2["lap_opts"]))
    with E.Context(p, E.ECS_PREC_FP64) as ctx:
        ctx.moments = np.zeros((1, p.Ny, p.Nx, 4))
        ctx.compute_rhs()
        b = ctx.rhs
        ctx.compute_lhs()
        x = np.random.default_rng(5).standard_normal(b.shape)
        y = ctx.lhs_apply(x)
    assert np.abs(b - g2["lap_rhs"]).max() <= 1e-15 * np.abs(g2["lap_rhs"]).max()
    y_ref = (g2["lap_lhs"] @ x.ravel()).reshape(x.shape)
    assert np.abs(y - y_ref).max() <= 1e-13 * np.abs(y_ref).max()


def test_mixed_push_move_deposit(built, g2):
    dt = float(g2["dt"])
    p = E.params_from_options(g2["opts"])
    with ctx_for(g2, E.ECS_PREC_MIXED) as ctx:
        ctx.upload_particles(g2["pos0"], g2["vel0"])
        ctx.phi = g2["phi"]
        ctx.push(dt)
        _, vel = ctx.download_particles()
        assert np.abs(vel - g2["vel_push"]).max() <= 2e-6 * np.abs(g2["vel_push"]).max()
        ctx.upload_particles(g2["pos0"], g2["vel_push"])
        ctx.update_positions(dt)
        pos, _ = ctx.download_particles()
        ctx.upload_particles(g2["pos_move"], g2["vel_move"])
        ctx.collect()
        m = ctx.moments
    cell = np.array([p.dx, p.dy])
    d = np.abs(pos - g2["pos_move"]) / cell
    d = np.minimum(d, np.array([p.Nx, p.Ny]) - d)  # across a periodic bound
    assert d.max() <= 2e-6
    ref = g2["moments"][..., 0]
    assert np.abs(m[..., 0] - ref).max() <= 1e-6 * np.abs(ref).max()


@pytest.mark.parametrize("prec", [E.ECS_PREC_FP64, E.ECS_PREC_MIXED])
def test_steps_256x256(built, prec):
    """256 x 256, 16 ions per cell from the device's Sobol initialiser, a few
    full steps (push, move, deposit, RHS, operator, multigrid solve coarsening
    x and y): ions kept, density sums to the ion count, solves reach 1e-8."""
    n = 256
    p = E.params_from_options(f"-ndim 2 -Nx {n} -Ny {n} -dx 1 -dy 1 -qi 1 -mi 1 -B0 0.1 -viT 1 -vi0x 1.0 "
                              "-nue 8.79e9 -Te 11604.5 -E0 0 -mn 0")
    N = n * n * 16
    with E.Context(p, prec, np_capacity=N) as ctx:
        ctx.init_particles(E.ECS_INIT_SOBOL, N)
        ctx.collect()
        st0 = ctx.compute_potential(rtol=1e-8, max_it=300)
        for _ in range(3):
            st = ctx.step(0.1, 1e-8, 300)
            assert st.solve.relres <= 1e-8
        m = ctx.moments
        assert int(E._lib.gpu().ecs_particles_count(ctx.handle)) == N
    assert abs(m[..., 0].sum() - N) <= 1e-9 * N
    print(f"prec {prec}: first solve {st0.iterations} its, step solve {st.solve.iterations} its "
          f"{1e3 * st.solve.seconds:.2f} ms, particles {1e3 * st.particle_seconds:.3f} ms")


def test_collisions_refused_in_2d(built, g2):
    p = E.params_from_options(g2["opts"].replace("-mn 0", ""))
    with pytest.raises(E.EcsError) as ei:
        E.Context(p, E.ECS_PREC_MIXED, np_capacity=10)
    assert ei.value.code == E._lib.ECS_ERR_UNSUPPORTED
