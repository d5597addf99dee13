"""GPU parity of the other operator options: -lhs identity / laplacian and
-rhs constant / sinusoidal (src/lhs.c:11-191, src/rhs.c:6-148).

Tolerances:
  RHS constant             bit-exact
  RHS sinusoidal           <= 1e-15 x max|b| (cos evaluated by CUDA's libm
                           against the reference's; the mean removal sums in
                           a different order)
  operator apply           <= 1e-14 relative against the reference's assembled
                           matrix (the Laplacian diagonal is summed in another
                           order)
  identity solve           phi = b, bit for bit
  Laplacian solves         relres <= rtol, re-measured with the reference's
                           matrix; on a periodic grid the cell-centred
                           cos(2 pi x) cos(2 pi y) cos(2 pi z) is an
                           eigenvector, so phi = b / lambda to 1e-7 relative
                           (mixed) / 1e-10 (FP64)
"""
import json

import numpy as np
import pytest

import ecsprt_gb300 as E
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

VARIANTS = ("lap_sin", "lap_const_zrefl", "id_const", "full_sin")


@pytest.fixture(scope="module")
def ops():
    return np.load(GOLDEN / "ops.npz")


def ctx_for(ops, variant, prec):
    opts = str(ops["opts_base"]) + json.loads(str(ops["variants"]))[variant]
    p = E.params_from_options(opts)
    ctx = E.Context(p, prec)
    dens = ops["full_sin_density"] if variant == "full_sin" else np.zeros((p.Nz, p.Ny, p.Nx))
    m = np.zeros(dens.shape + (4,))
    m[..., 0] = dens
    ctx.moments = m
    return ctx


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("prec", [E.ECS_PREC_FP64, E.ECS_PREC_MIXED])
def test_rhs_and_operator(built, ops, variant, prec):
    b_ref = ops[f"{variant}_rhs"]
    A = ops[f"{variant}_lhs"]
    with ctx_for(ops, variant, prec) as ctx:
        ctx.compute_rhs()
        b = ctx.rhs
        ctx.compute_lhs()
        x = np.random.default_rng(3).standard_normal(b.shape)
        y = ctx.lhs_apply(x)
    if variant.endswith("const") or "const_" in variant:
        assert np.array_equal(b, b_ref)
    else:
        assert np.abs(b - b_ref).max() <= 1e-15 * np.abs(b_ref).max()
    y_ref = (A @ x.ravel()).reshape(x.shape)
    assert np.abs(y - y_ref).max() <= 1e-14 * max(np.abs(y_ref).max(), 1.0)


@pytest.mark.parametrize("prec", [E.ECS_PREC_FP64, E.ECS_PREC_MIXED])
def test_identity_solve(built, ops, prec):
    with ctx_for(ops, "id_const", prec) as ctx:
        st = ctx.compute_potential(rtol=1e-8, max_it=50)
        phi, b = ctx.phi, ctx.rhs
    assert np.array_equal(phi, b)
    assert st.relres == 0.0 and st.iterations == 0


@pytest.mark.parametrize("variant", ["lap_sin", "lap_const_zrefl"])
@pytest.mark.parametrize("prec", [E.ECS_PREC_FP64, E.ECS_PREC_MIXED])
def test_laplacian_solve_small(built, ops, variant, prec):
    rtol = 1e-11 if prec == E.ECS_PREC_FP64 else 1e-8
    A = ops[f"{variant}_lhs"]
    with ctx_for(ops, variant, prec) as ctx:
        st = ctx.compute_potential(rtol=rtol, max_it=200)
        phi, b = ctx.phi, ctx.rhs
    r = b.ravel() - A @ phi.ravel()
    assert st.relres <= rtol
    assert np.linalg.norm(r) / np.linalg.norm(b) <= 2 * rtol


@pytest.mark.parametrize("prec", [E.ECS_PREC_FP64, E.ECS_PREC_MIXED])
def test_laplacian_sinusoid_eigenvector(built, prec):
    """64^3 periodic, dx = 1/64: the sinusoidal RHS is one Fourier mode and the
    discrete Laplacian's eigenvalue is sum_d (2 cos(2 pi h) - 2) / h^2."""
    n = 64
    h = 1.0 / n
    p = E.params_from_options(f"-Nx {n} -Ny {n} -Nz {n} -dx {h} -dy {h} -dz {h} -n0 1.5 -lhs laplacian "
                              f"-rhs sinusoidal -qi 1 -mi 1 -B0 0.1 -nue 8.79e9 -Te 11604.5")
    rtol = 1e-11 if prec == E.ECS_PREC_FP64 else 1e-8
    with E.Context(p, prec) as ctx:
        ctx.moments = np.zeros((n, n, n, 4))
        st = ctx.compute_potential(rtol=rtol, max_it=200)
        phi, b = ctx.phi, ctx.rhs
    lam = 3 * (2 * np.cos(2 * np.pi * h) - 2) / (h * h)
    assert st.relres <= rtol
    tol = 1e-10 if prec == E.ECS_PREC_FP64 else 1e-7
    assert np.linalg.norm(phi - b / lam) <= tol * np.linalg.norm(b / lam)
    print(f"prec {prec}: {st.iterations} iterations, {st.refinements} refinements, {1e3 * st.seconds:.2f} ms")


def test_constant_rhs_periodic_laplacian_is_inconsistent(built, ops):
    """A constant RHS against the periodic Laplacian's constant null space has
    no solution: the solve reports non-convergence instead of a potential."""
    opts = str(ops["opts_base"]) + "-lhs laplacian -rhs constant"
    p = E.params_from_options(opts)
    with E.Context(p, E.ECS_PREC_MIXED) as ctx:
        ctx.moments = np.zeros((p.Nz, p.Ny, p.Nx, 4))
        with pytest.raises(E.EcsError) as ei:
            ctx.compute_potential(rtol=1e-8, max_it=40)
    assert ei.value.code == E._lib.ECS_ERR_NOT_CONVERGED


def test_served_laplacian_matches_context(built):
    """The request graph of the server runs the option variants too."""
    n = 32
    p = E.params_from_options(f"-Nx {n} -Ny {n} -Nz {n} -dx {1 / n} -dy {1 / n} -dz {1 / n} -n0 2 "
                              "-lhs laplacian -rhs sinusoidal -qi 1 -mi 1 -B0 0.1 -nue 8.79e9 -Te 11604.5")
    d = np.ones((n, n, n))
    with E.Context(p, E.ECS_PREC_MIXED) as ctx:
        phi0, _ = ctx.solve_density(d, rtol=1e-8, max_it=200)
    with E.Server(hbm_budget_bytes=1 << 30, max_inflight=2) as srv:
        out = np.empty_like(d)
        srv.submit_solve(p, d, out)
        res = srv.wait_all(60)
    assert res[0]["status"] == 0
    assert np.array_equal(out, phi0)
